// Allocation-free variant of the FP64 RI JK build (gb_jkj_ri_noalloc_f64).
//
// Who needs it: callers that may not allocate device memory on their own --
// for example a process whose HBM is owned entirely by another allocator (a
// framework's caching pool, or a fixed arena reserved at start-up so that work
// can be admitted against an HBM budget), where an extra cudaMalloc would fail
// or fragment that budget, and latency-critical loops where cudaMalloc and
// cudaFree would synchronise the device.  Such callers still supply inputs and
// outputs, but cannot hand the library a workspace.
//
// How: the scratch is a file-scope __device__ array of fixed size.  The CUDA
// driver reserves it on every GPU where this library's module is loaded and it
// stays reserved until the process exits.  Host code cannot use the array's
// name as a device address (on the host it names a host-side stand-in), so the
// device address is looked up with cudaGetSymbolAddress, with the device
// current, and passed to the kernels as a plain pointer.  The address is
// cached per device together with the id of the context it belongs to; a
// context created anew (after cudaDeviceReset) has a new id and the next call
// looks the address up again.
//
// The first call on each device (and the first after a cudaDeviceReset)
// performs that lookup, which may also load the module on that device; make
// that call before any stream capture.
//
// Every call on a device uses the same array, and the array keeps whatever the
// previous call left in it.  No part of it needs clearing: every scratch
// element the build reads is written earlier in the same call.  Calls whose
// execution overlaps on the GPU (different streams, or different host threads
// without ordering) race on the array and produce wrong results: serialise
// them on one stream.
#include <mutex>

#include "gb_common.cuh"

static __device__ __align__(256) unsigned char g_noalloc_scratch[GB_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};  // context id the cached address belongs to

// Device address of g_noalloc_scratch on the current device (looked up once
// per device context).
int scratch_address(void** out) {
  int dev = -1;
  GB_TRY(gb::cuda_status(cudaGetDevice(&dev), "gb_jkj_ri_noalloc_f64: cudaGetDevice"));
  GB_REQUIRE(dev >= 0 && dev < kMaxDevices, GB_ERR_UNSUPPORTED,
             "gb_jkj_ri_noalloc_f64: device ordinal %d beyond %d", dev, kMaxDevices);
  const unsigned long long ctx = gb::current_context_id();
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_scratch_addr[dev] == nullptr || ctx == 0 || g_scratch_ctx[dev] != ctx) {
    void* p = nullptr;
    GB_TRY(gb::cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                           "gb_jkj_ri_noalloc_f64: cudaGetSymbolAddress"));
    GB_REQUIRE(p != nullptr, GB_ERR_CUDA, "gb_jkj_ri_noalloc_f64: null scratch address");
    g_scratch_addr[dev] = p;
    g_scratch_ctx[dev] = gb::current_context_id();
  }
  *out = g_scratch_addr[dev];
  return GB_OK;
}

}  // namespace

extern "C" int gb_jkj_ri_noalloc_f64(const double* C, const double* b, int nbf, int nbf5, int naux, double* J,
                                     double* K, void* stream) {
  gb::clear_error();
  if (nbf <= 0 || nbf5 <= 0 || naux <= 0 || nbf5 > nbf) {
    // invalid sizes: the regular entry point reports them before touching scratch
    return gb_jkj_ri_f64(C, b, nbf, nbf5, naux, J, K, nullptr, 0, stream);
  }
  const size_t need = gb_jkj_ri_workspace_f64(nbf, nbf5, naux);
  GB_REQUIRE(need <= (size_t)GB_NOALLOC_SCRATCH_BYTES, GB_ERR_WORKSPACE,
             "gb_jkj_ri_noalloc_f64: nbf=%d nbf5=%d naux=%d needs %zu bytes of scratch, more than the "
             "%zu-byte built-in scratch (nbf5*nbf*naux + nbf5*naux doubles must fit); use gb_jkj_ri_f64 with "
             "a caller workspace",
             nbf, nbf5, naux, need, (size_t)GB_NOALLOC_SCRATCH_BYTES);
  void* scratch = nullptr;
  GB_TRY(scratch_address(&scratch));
  return gb_jkj_ri_f64(C, b, nbf, nbf5, naux, J, K, scratch, (size_t)GB_NOALLOC_SCRATCH_BYTES, stream);
}
