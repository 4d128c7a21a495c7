// Status reporting and small utility entry points of the C ABI.
#include <cstdarg>
#include <cstdio>
#include <new>

#include "gb_common.cuh"

namespace gb {

static thread_local char g_last_error[1024] = "";

void set_error(int code, const char* fmt, ...) {
  char msg[900];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof(msg), fmt, ap);
  va_end(ap);
  snprintf(g_last_error, sizeof(g_last_error), "[GB status %d] %s", code, msg);
}

void clear_error() { g_last_error[0] = '\0'; }

namespace {

__global__ void symmetric_diff_kernel(const double* __restrict__ b, int N, int Q, unsigned long long* out) {
  // warps stride over the (m, n) index pairs and keep the pairs with n > m; the
  // maximum |b[m][n][l] - b[n][m][l]| is folded with an atomicMax on the bit
  // pattern (order-preserving for non-negative doubles)
  double mx = 0.0;
  const long long total = (long long)N * N;
  for (long long t = (long long)blockIdx.x * blockDim.y + threadIdx.y; t < total;
       t += (long long)gridDim.x * blockDim.y) {
    const long long m = t / N, n = t % N;
    if (n <= m) continue;
    const double* x = b + (m * N + n) * Q;
    const double* y = b + (n * N + m) * Q;
    for (int l = threadIdx.x; l < Q; l += blockDim.x) mx = fmax(mx, fabs(x[l] - y[l]));
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (threadIdx.x == 0) atomicMax(out, (unsigned long long)__double_as_longlong(mx));
}

}  // namespace
}  // namespace gb

extern "C" const char* gb_last_error(void) { return gb::g_last_error; }

extern "C" int gb_version(void) { return 100; }

extern "C" int gb_check_symmetric_f64(const double* b, int nbf, int naux, double* max_abs_diff, void* stream) {
  gb::clear_error();
  GB_REQUIRE(b && max_abs_diff, GB_ERR_INVALID_ARG, "gb_check_symmetric_f64: null pointer");
  GB_REQUIRE(nbf > 0 && naux > 0, GB_ERR_BAD_SHAPE, "gb_check_symmetric_f64: bad sizes");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GB_TRY(gb::cuda_status(cudaMemsetAsync(max_abs_diff, 0, sizeof(double), s), "gb_check_symmetric_f64"));
  if (nbf == 1) return GB_OK;
  gb::symmetric_diff_kernel<<<1024, dim3(32, 8), 0, s>>>(b, nbf, naux,
                                                         reinterpret_cast<unsigned long long*>(max_abs_diff));
  GB_CHECK_LAUNCH("symmetric_diff");
  return GB_OK;
}

// ---------------------------------------------------------------------------
// Capture of a caller's stream work into a CUDA graph (thread-local mode, so
// other threads' CUDA calls are not affected while a capture is open).
// ---------------------------------------------------------------------------
using gb::clear_error;
using gb::cuda_status;
using gb::set_error;

struct gb_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

extern "C" int gb_graph_begin(void* stream) {
  clear_error();
  GB_REQUIRE(stream, GB_ERR_INVALID_ARG, "gb_graph_begin: capture needs a non-default stream");
  return cuda_status(cudaStreamBeginCapture(static_cast<cudaStream_t>(stream), cudaStreamCaptureModeThreadLocal),
                     "cudaStreamBeginCapture");
}

extern "C" int gb_graph_end(void* stream, gb_graph** out) {
  clear_error();
  GB_REQUIRE(stream && out, GB_ERR_INVALID_ARG, "gb_graph_end: null argument");
  cudaGraph_t g = nullptr;
  GB_TRY(cuda_status(cudaStreamEndCapture(static_cast<cudaStream_t>(stream), &g), "cudaStreamEndCapture"));
  cudaGraphExec_t e = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&e, g, 0);
  if (ei != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_status(ei, "cudaGraphInstantiate");
  }
  gb_graph* h = new (std::nothrow) gb_graph;
  if (!h) {
    cudaGraphExecDestroy(e);
    cudaGraphDestroy(g);
    set_error(GB_ERR_INVALID_ARG, "gb_graph_end: out of host memory");
    return GB_ERR_INVALID_ARG;
  }
  h->graph = g;
  h->exec = e;
  *out = h;
  return GB_OK;
}

extern "C" int gb_graph_launch(gb_graph* g, void* stream) {
  clear_error();
  GB_REQUIRE(g && g->exec, GB_ERR_INVALID_ARG, "gb_graph_launch: no graph");
  return cuda_status(cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(stream)), "cudaGraphLaunch");
}

extern "C" int gb_graph_destroy(gb_graph* g) {
  clear_error();
  if (!g) return GB_OK;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
  return GB_OK;
}

