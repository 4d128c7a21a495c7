// Orbital rotation C' = C expm(Y) on the device, FP64 (rotate_orbital,
// utils.py:550-565): Y is the antisymmetric matrix whose strict upper
// triangle, rows i < nbf5, holds the packed step y (row-major over (i, j > i),
// the order of numpy's triu_indices(nbf, 1) restricted to i < nbf5).
//
// expm by scaling and squaring: X = Y / 2^s with ||X||_1 <= 1/2, the degree-16
// Taylor polynomial of X (truncation < 0.5^17 / 17! ~ 2e-20 relative), then s
// squarings.  The polynomial is evaluated Paterson-Stockmeyer style in X^4:
//   p(X) = B0 + X^4 (B1 + X^4 (B2 + X^4 (B3 + X^4 B4))),  Bj = sum_i c_{4j+i} X^i
// with c_k = 1/k!: X^2, X^3, X^4 and three Horner products are six GEMMs on
// the DMMA engine, plus s squarings and the final C U.
#include <cmath>
#include <cstring>

#include "gemm_f64.cuh"

using namespace gb;

namespace {

constexpr int TAYLOR_DEG = 16;

// Y[i][j] from the packed step: +y for i < j (i < P), -y for i > j (j < P).
__global__ void build_antisym_kernel(const double* __restrict__ y, int N, int P, double* __restrict__ Y) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)N * N) return;
  const int i = (int)(idx / N), j = (int)(idx % N);
  double v = 0.0;
  const int lo = i < j ? i : j, hi = i < j ? j : i;
  if (lo != hi && lo < P) {
    // offset of row lo in the packed upper triangle: sum_{r < lo} (N - 1 - r)
    const long long off = (long long)lo * (N - 1) - (long long)lo * (lo - 1) / 2;
    v = y[off + (hi - lo - 1)];
    if (i > j) v = -v;
  }
  Y[idx] = v;
}

// norm[0] = max_j sum_i |Y[i][j]| (bit-pattern max: non-negative doubles order as integers)
__global__ void col_abs_max_kernel(const double* __restrict__ Y, int N, unsigned long long* __restrict__ norm) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  double s = 0.0;
  for (int i = 0; i < N; ++i) s += fabs(Y[(long long)i * N + j]);
  atomicMax(norm, (unsigned long long)__double_as_longlong(s));
}

// dst = sum_{i<4} c[i] X^i (X^0 = I) + c4 X4 (X4 may be null), X^i scaled by `scale` first
__global__ void poly_block_kernel(double* __restrict__ dst, const double* __restrict__ X1,
                                  const double* __restrict__ X2, const double* __restrict__ X3,
                                  const double* __restrict__ X4, int N, double c0, double c1, double c2, double c3,
                                  double c4) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)N * N) return;
  const int i = (int)(idx / N), j = (int)(idx % N);
  double v = (i == j) ? c0 : 0.0;
  v = fma(c1, X1[idx], v);
  v = fma(c2, X2[idx], v);
  v = fma(c3, X3[idx], v);
  if (X4) v = fma(c4, X4[idx], v);
  dst[idx] = v;
}

__global__ void scale_kernel(const double* __restrict__ src, double* __restrict__ dst, long long n, double f) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < n) dst[idx] = src[idx] * f;
}

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// C = A B (+ C when accumulate), square row-major N x N
int matmul(const double* A, const double* B, double* C, int N, bool accumulate, cudaStream_t s, const char* tag) {
  GemmF64 g{};
  g.M = N; g.N = N; g.K = N; g.batch = 1;
  g.A = {A, 0, lin(N), lin(1)};
  g.B = {B, 0, lin(N), lin(1)};
  g.C = {C, 0, lin(N), lin(1)};
  g.alpha = 1.0; g.beta = accumulate ? 1.0 : 0.0; g.sym = SYM_NONE;
  g.a_kfast = true; g.b_kfast = false;
  g.tag = tag;
  return gemm_f64(g, s);
}

template <class Cv>
void rotate_layout(Cv& c, int N, double** bufs, unsigned long long** norm) {
  for (int k = 0; k < 6; ++k) {
    double* p = c.template take<double>((size_t)N * N);
    if (bufs) bufs[k] = p;
  }
  auto* nm = c.template take<unsigned long long>(1);
  if (norm) *norm = nm;
}

}  // namespace

extern "C" size_t gb_rotate_orbital_workspace_f64(int nbf) {
  SizeCarve c;
  rotate_layout(c, nbf, nullptr, nullptr);
  return c.used;
}

extern "C" int gb_rotate_orbital_f64(const double* y, const double* C, int nbf, int nbf5, double norm1,
                                     double* Cout, void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5;
  GB_REQUIRE(N > 0 && P > 0 && P <= N, GB_ERR_BAD_SHAPE, "gb_rotate_orbital_f64: need 0 < nbf5 <= nbf");
  GB_REQUIRE(y && C && Cout, GB_ERR_INVALID_ARG, "gb_rotate_orbital_f64: null pointer");
  GB_REQUIRE(C != Cout, GB_ERR_INVALID_ARG, "gb_rotate_orbital_f64: C and Cout must not alias");
  GB_REQUIRE(workspace_bytes >= gb_rotate_orbital_workspace_f64(N), GB_ERR_WORKSPACE,
             "gb_rotate_orbital_f64: workspace too small");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Carve wc(workspace, workspace_bytes);
  double* buf[6];
  unsigned long long* dnorm = nullptr;
  rotate_layout(wc, N, buf, &dnorm);
  double *Y = buf[0], *X2 = buf[1], *X3 = buf[2], *X4 = buf[3], *R0 = buf[4], *R1 = buf[5];
  const long long NN = (long long)N * N;

  GB_LAUNCH("rotate_build", s, build_antisym_kernel<<<cdiv(NN, 256), 256, 0, s>>>(y, N, P, Y));
  double norm = norm1;
  if (!(norm1 >= 0.0)) {
    // no bound from the caller: measure ||Y||_1 on the device (one synchronisation)
    GB_TRY(cuda_status(cudaMemsetAsync(dnorm, 0, sizeof(unsigned long long), s), "cudaMemsetAsync"));
    GB_LAUNCH("rotate_norm", s, col_abs_max_kernel<<<cdiv(N, 128), 128, 0, s>>>(Y, N, dnorm));
    unsigned long long nbits = 0;
    GB_TRY(cuda_status(cudaMemcpyAsync(&nbits, dnorm, sizeof(nbits), cudaMemcpyDeviceToHost, s), "norm copy"));
    GB_TRY(cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize"));
    memcpy(&norm, &nbits, sizeof(norm));
  }
  GB_REQUIRE(std::isfinite(norm), GB_ERR_NONFINITE, "gb_rotate_orbital_f64: step y is not finite");
  GB_REQUIRE(norm < 0x1p60, GB_ERR_INVALID_ARG, "gb_rotate_orbital_f64: step norm %g too large", norm);
  int sq = 0;
  while (norm > 0.5) {
    norm *= 0.5;
    ++sq;
  }
  // X = Y / 2^sq in place
  if (sq > 0)
    GB_LAUNCH("rotate_scale", s, scale_kernel<<<cdiv(NN, 256), 256, 0, s>>>(Y, Y, NN, std::ldexp(1.0, -sq)));
  const double* X = Y;
  double c[TAYLOR_DEG + 1];
  c[0] = 1.0;
  for (int k = 1; k <= TAYLOR_DEG; ++k) c[k] = c[k - 1] / k;
  GB_TRY(matmul(X, X, X2, N, false, s, "gemm_f64:expm"));
  GB_TRY(matmul(X2, X, X3, N, false, s, "gemm_f64:expm"));
  GB_TRY(matmul(X2, X2, X4, N, false, s, "gemm_f64:expm"));
  // R = B3 + c16 X^4
  GB_LAUNCH("rotate_poly", s,
            poly_block_kernel<<<cdiv(NN, 256), 256, 0, s>>>(R0, X, X2, X3, X4, N, c[12], c[13], c[14], c[15],
                                                              c[16]));
  double *R = R0, *Rn = R1;
  for (int j = 2; j >= 0; --j) {
    // Rn = Bj + X^4 R
    GB_LAUNCH("rotate_poly", s,
              poly_block_kernel<<<cdiv(NN, 256), 256, 0, s>>>(Rn, X, X2, X3, nullptr, N, c[4 * j], c[4 * j + 1],
                                                                c[4 * j + 2], c[4 * j + 3], 0.0));
    GB_TRY(matmul(X4, R, Rn, N, true, s, "gemm_f64:expm"));
    double* t = R;
    R = Rn;
    Rn = t;
  }
  // s squarings, ping-ponging between R and a free buffer
  double* spare = X2;
  for (int k = 0; k < sq; ++k) {
    GB_TRY(matmul(R, R, spare, N, false, s, "gemm_f64:expm"));
    double* t = R;
    R = spare;
    spare = t;
  }
  return matmul(C, R, Cout, N, false, s, "gemm_f64:rotate");
}
