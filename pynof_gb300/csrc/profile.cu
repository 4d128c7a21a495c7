// Optional launch profiler: when enabled, every internal kernel launch is
// bracketed by a pair of CUDA events on its own stream, so the host can read
// per-kernel device time over a region without an external profiler.
// Disabled by default; the disabled cost is one relaxed atomic load per launch.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "gb_common.cuh"

namespace gb {
namespace {

struct Rec {
  const char* name;
  cudaEvent_t a, b;
};

std::atomic<bool> g_on{false};
std::mutex g_mu;
std::vector<Rec> g_recs;

}  // namespace

int prof_begin(const char* name, cudaStream_t s) {
  if (!g_on.load(std::memory_order_relaxed)) return -1;
  Rec r{name, nullptr, nullptr};
  if (cudaEventCreate(&r.a) != cudaSuccess || cudaEventCreate(&r.b) != cudaSuccess) return -1;
  cudaEventRecord(r.a, s);
  std::lock_guard<std::mutex> lk(g_mu);
  g_recs.push_back(r);
  return (int)g_recs.size() - 1;
}

void prof_end(int idx, cudaStream_t s) {
  if (idx < 0) return;
  std::lock_guard<std::mutex> lk(g_mu);
  if (idx < (int)g_recs.size()) cudaEventRecord(g_recs[idx].b, s);
}

}  // namespace gb

extern "C" int gb_profile_start(void) {
  gb::clear_error();
  std::lock_guard<std::mutex> lk(gb::g_mu);
  for (auto& r : gb::g_recs) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  gb::g_recs.clear();
  gb::g_on.store(true);
  return GB_OK;
}

extern "C" int gb_profile_stop(char* out, size_t out_len) {
  gb::clear_error();
  gb::g_on.store(false);
  std::lock_guard<std::mutex> lk(gb::g_mu);
  std::map<std::string, std::pair<long, double>> agg;
  int status = GB_OK;
  for (auto& r : gb::g_recs) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess)
      status = GB_ERR_CUDA;
    auto& e = agg[r.name];
    e.first += 1;
    e.second += ms;
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  gb::g_recs.clear();
  std::string js = "{";
  bool first = true;
  for (auto& kv : agg) {
    char buf[256];
    snprintf(buf, sizeof(buf), "%s\"%s\": [%ld, %.6f]", first ? "" : ", ", kv.first.c_str(), kv.second.first,
             kv.second.second);
    js += buf;
    first = false;
  }
  js += "}";
  if (out && out_len) {
    if (js.size() + 1 > out_len) {
      gb::set_error(GB_ERR_INVALID_ARG, "gb_profile_stop: buffer too small (%zu needed)", js.size() + 1);
      return GB_ERR_INVALID_ARG;
    }
    memcpy(out, js.c_str(), js.size() + 1);
  }
  if (status != GB_OK) gb::set_error(status, "gb_profile_stop: event query failed");
  return status;
}
