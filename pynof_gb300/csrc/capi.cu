// Status reporting and small utility entry points of the C ABI.
#include <cstdarg>
#include <cstdio>

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
