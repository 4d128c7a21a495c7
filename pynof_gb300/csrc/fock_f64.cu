// Generalized Fock matrices, the Lagrangian from them and the electronic
// energy (FP64): computeF_RC, computeF_RO, computeLagrange, computeE_elec.
#include "gemm_f64.cuh"
#include "ri_kernels.cuh"

using namespace gb;

namespace {

// dst = src with the diagonal entries (i, i), i >= ini, set to zero.
__global__ void zero_diag_from_kernel(const double* __restrict__ src, double* __restrict__ dst, int P, int ini) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)P * P) return;
  const int r = (int)(idx / P), c = (int)(idx % P);
  dst[idx] = (r == c && r >= ini) ? 0.0 : src[idx];
}

// F[i] += n_i H + coef_i n_i J_i,  coef_i = 1 for ini <= i < nbeta and nalpha <= i < P
__global__ void fock_diag_terms_kernel(double* __restrict__ F, const double* __restrict__ J,
                                       const double* __restrict__ H, const double* __restrict__ n, int N, int P,
                                       int ini, int nbeta, int nalpha) {
  const long long mn = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  const long long NN = (long long)N * N;
  if (mn >= NN) return;
  const double ni = n[i];
  const bool cj = (i >= ini && i < nbeta) || (i >= nalpha && i < P);
  const long long o = (long long)i * NN + mn;
  double v = F[o] + ni * H[mn];
  if (cj) v += ni * J[o];
  F[o] = v;
}

// Coupling coefficients of the restricted open-shell generalized Fock
//   F_i = a_i H + sum_j A[i][j] J_j - sum_j B[i][j] K_j
// with D = [0, nbeta) u [nalpha, P) (doubly occupied and correlating) and
// O = [nbeta, nalpha) (singly occupied):
//   a_i = n_i on D, 1/2 on O;
//   A[i][j] = cj12[i][j] (i, j in D; diagonal from ini on zero)
//           + n_i (i == j, i in [ini, nbeta) or [nalpha, P))
//           + n_i (i in D, j in O) + 1/2 (i, j in O, i != j) + n_j (i in O, j in D)
//   B[i][j] = ck12[i][j] (i, j in D; diagonal from ini on zero)
//           + n_i / 2 (i in D, j in O) + 1/2 (i, j in O, i != j) + n_j / 2 (i in O, j in D)
// One thread per (i, j); the (i, 0) threads also write a_i.
__global__ void fock_ro_coef_kernel(const double* __restrict__ n, const double* __restrict__ cj12,
                                    const double* __restrict__ ck12, double* __restrict__ A, double* __restrict__ B,
                                    double* __restrict__ a, int P, int ini, int nbeta, int nalpha) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)P * P) return;
  const int i = (int)(idx / P), j = (int)(idx % P);
  const bool oi = i >= nbeta && i < nalpha, oj = j >= nbeta && j < nalpha;
  double av = 0.0, bv = 0.0;
  if (!oi && !oj) {
    const bool zero = (i == j && i >= ini);
    av = zero ? 0.0 : cj12[idx];
    bv = zero ? 0.0 : ck12[idx];
    if (i == j && ((i >= ini && i < nbeta) || i >= nalpha)) av += n[i];
  } else if (!oi && oj) {
    av = n[i];
    bv = 0.5 * n[i];
  } else if (oi && oj) {
    av = i != j ? 0.5 : 0.0;
    bv = av;
  } else {
    av = n[j];
    bv = 0.5 * n[j];
  }
  A[idx] = av;
  B[idx] = bv;
  if (j == 0) a[i] = oi ? 0.5 : n[i];
}

// F[i] += a_i H
__global__ void fock_add_h_kernel(double* __restrict__ F, const double* __restrict__ H, const double* __restrict__ a,
                                  int N) {
  const long long mn = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  const long long NN = (long long)N * N;
  if (mn >= NN) return;
  const long long o = (long long)i * NN + mn;
  F[o] = fma(a[i], H[mn], F[o]);
}

// G[i][m] = sum_n F[i][m][n] C[n][i]   (one warp per (i, m))
__global__ void fock_times_orbital_kernel(const double* __restrict__ F, const double* __restrict__ C,
                                          double* __restrict__ G, int N, int P) {
  const long long w = (long long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= (long long)P * N) return;
  const int i = (int)(w / N), m = (int)(w % N);
  const double* f = F + ((long long)i * N + m) * N;
  double acc = 0.0;
  for (int nn = lane; nn < N; nn += 32) acc = fma(f[nn], C[(long long)nn * N + i], acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) G[(long long)i * N + m] = acc;
}

__global__ void zero_outside_kernel(double* __restrict__ elag, int N, int rows, int cols) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)N * N) return;
  const int r = (int)(idx / N), c = (int)(idx % N);
  if (r >= rows || c >= cols) elag[idx] = 0.0;
}

// E = tr(elag[:P,:P]) + sum_i w_i Hd_i with w_i = n_i (or 1/2 for singly occupied
// orbitals when high_spin); single block
__global__ void energy_elec_kernel(const double* __restrict__ elag, const double* __restrict__ Hd,
                                   const double* __restrict__ n, int N, int P, int nbeta, int nalpha, int high_spin,
                                   double* __restrict__ E) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    double w = n[i];
    if (high_spin && i >= nbeta && i < nalpha) w = 0.5;
    acc += elag[(long long)i * N + i] + w * Hd[i];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) *E = v;
  }
}

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

// ---------------------------------------------------------------------------
// A8  computeF_RC (closed shell)
// ---------------------------------------------------------------------------
extern "C" size_t gb_fock_rc_workspace_f64(int nbf, int nbf5) {
  Sizer z;
  z.add<double>((size_t)nbf5 * nbf5);
  z.add<double>((size_t)nbf5 * nbf5);
  (void)nbf;
  return z.used;
}

extern "C" int gb_fock_rc_f64(const double* J, const double* K, const double* n, const double* H,
                              const double* cj12, const double* ck12, int nbf, int nbf5, int nbeta, int nalpha,
                              int no1, double* F, void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5;
  GB_REQUIRE(N > 0 && P > 0 && P <= N, GB_ERR_BAD_SHAPE, "gb_fock_rc_f64: bad sizes nbf=%d nbf5=%d", N, P);
  GB_REQUIRE(0 <= nbeta && nbeta <= nalpha && nalpha <= P && no1 >= 0, GB_ERR_BAD_SHAPE,
             "gb_fock_rc_f64: need 0 <= nbeta <= nalpha <= nbf5");
  GB_REQUIRE(J && K && n && H && cj12 && ck12 && F, GB_ERR_INVALID_ARG, "gb_fock_rc_f64: null pointer");
  Carve cv(workspace, workspace_bytes);
  double* cjm = cv.take<double>((size_t)P * P);
  double* ckm = cv.take<double>((size_t)P * P);
  GB_REQUIRE(cjm && ckm, GB_ERR_WORKSPACE, "gb_fock_rc_f64: workspace too small");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int ini = no1 > 1 ? no1 : 0;
  GB_LAUNCH("zero_diag_from", s, zero_diag_from_kernel<<<cdiv((long long)P * P, 256), 256, 0, s>>>(cj12, cjm, P, ini));
  GB_LAUNCH("zero_diag_from", s, zero_diag_from_kernel<<<cdiv((long long)P * P, 256), 256, 0, s>>>(ck12, ckm, P, ini));
  const long long NN = (long long)N * N;
  // F = cj12' J
  GemmF64 g{};
  g.M = P; g.N = (int)NN; g.K = P; g.batch = 1;
  g.A = {cjm, 0, lin(P), lin(1)};
  g.B = {J, 0, lin(NN), lin(1)};
  g.C = {F, 0, lin(NN), lin(1)};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_NONE;
  g.a_kfast = true; g.b_kfast = false;
  g.tag = "gemm_f64:fock";
  GB_TRY(gemm_f64(g, s));
  // F -= ck12' K
  g.A = {ckm, 0, lin(P), lin(1)};
  g.B = {K, 0, lin(NN), lin(1)};
  g.alpha = -1.0; g.beta = 1.0;
  GB_TRY(gemm_f64(g, s));
  GB_LAUNCH("fock_diag_terms", s,
            fock_diag_terms_kernel<<<dim3(cdiv(NN, 256), P), 256, 0, s>>>(F, J, H, n, N, P, ini, nbeta, nalpha));
  return GB_OK;
}

// ---------------------------------------------------------------------------
// A8  computeF_RO (restricted open shell)
// ---------------------------------------------------------------------------
extern "C" size_t gb_fock_ro_workspace_f64(int nbf, int nbf5) {
  Sizer z;
  z.add<double>((size_t)nbf5 * nbf5);
  z.add<double>((size_t)nbf5 * nbf5);
  z.add<double>((size_t)nbf5);
  (void)nbf;
  return z.used;
}

extern "C" int gb_fock_ro_f64(const double* J, const double* K, const double* n, const double* H,
                              const double* cj12, const double* ck12, int nbf, int nbf5, int nbeta, int nalpha,
                              int no1, double* F, void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5;
  GB_REQUIRE(N > 0 && P > 0 && P <= N, GB_ERR_BAD_SHAPE, "gb_fock_ro_f64: bad sizes nbf=%d nbf5=%d", N, P);
  GB_REQUIRE(0 <= nbeta && nbeta <= nalpha && nalpha <= P && no1 >= 0 && no1 <= nbeta, GB_ERR_BAD_SHAPE,
             "gb_fock_ro_f64: need 0 <= no1 <= nbeta <= nalpha <= nbf5");
  GB_REQUIRE(J && K && n && H && cj12 && ck12 && F, GB_ERR_INVALID_ARG, "gb_fock_ro_f64: null pointer");
  Carve cv(workspace, workspace_bytes);
  double* A = cv.take<double>((size_t)P * P);
  double* B = cv.take<double>((size_t)P * P);
  double* a = cv.take<double>((size_t)P);
  GB_REQUIRE(A && B && a, GB_ERR_WORKSPACE, "gb_fock_ro_f64: workspace too small");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int ini = no1 > 1 ? no1 : 0;
  GB_LAUNCH("fock_ro_coef", s,
            fock_ro_coef_kernel<<<cdiv((long long)P * P, 256), 256, 0, s>>>(n, cj12, ck12, A, B, a, P, ini, nbeta,
                                                                             nalpha));
  const long long NN = (long long)N * N;
  // F = A J - B K
  GemmF64 g{};
  g.M = P; g.N = (int)NN; g.K = P; g.batch = 1;
  g.A = {A, 0, lin(P), lin(1)};
  g.B = {J, 0, lin(NN), lin(1)};
  g.C = {F, 0, lin(NN), lin(1)};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_NONE;
  g.a_kfast = true; g.b_kfast = false;
  g.tag = "gemm_f64:fock";
  GB_TRY(gemm_f64(g, s));
  g.A = {B, 0, lin(P), lin(1)};
  g.B = {K, 0, lin(NN), lin(1)};
  g.alpha = -1.0; g.beta = 1.0;
  GB_TRY(gemm_f64(g, s));
  GB_LAUNCH("fock_add_h", s, fock_add_h_kernel<<<dim3(cdiv(NN, 256), P), 256, 0, s>>>(F, H, a, N));
  return GB_OK;
}

// ---------------------------------------------------------------------------
// A8  computeLagrange:  elag[:noptorb, :nbf5] = C^T G,  G[m][i] = F_i[m] . C_i
// ---------------------------------------------------------------------------
extern "C" size_t gb_lagrange_workspace_f64(int nbf, int nbf5) {
  Sizer z;
  z.add<double>((size_t)nbf5 * nbf);
  return z.used;
}

extern "C" int gb_lagrange_f64(const double* F, const double* C, int nbf, int nbf5, int noptorb, double* elag,
                               void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5;
  GB_REQUIRE(N > 0 && P > 0 && P <= N && noptorb > 0 && noptorb <= N, GB_ERR_BAD_SHAPE,
             "gb_lagrange_f64: bad sizes nbf=%d nbf5=%d noptorb=%d", N, P, noptorb);
  GB_REQUIRE(F && C && elag, GB_ERR_INVALID_ARG, "gb_lagrange_f64: null pointer");
  Carve cv(workspace, workspace_bytes);
  double* G = cv.take<double>((size_t)P * N);  // G[i][m]
  GB_REQUIRE(G, GB_ERR_WORKSPACE, "gb_lagrange_f64: workspace too small");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GB_LAUNCH("fock_times_orbital", s,
            fock_times_orbital_kernel<<<cdiv((long long)P * N, 8), 256, 0, s>>>(F, C, G, N, P));
  GemmF64 g{};
  g.M = noptorb; g.N = P; g.K = N; g.batch = 1;
  g.A = {C, 0, lin(1), lin(N)};   // A(k, m) = C[m][k]
  g.B = {G, 0, lin(1), lin(N)};   // B(m, i) = G[i][m]
  g.C = {elag, 0, lin(N), lin(1)};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_NONE;
  g.a_kfast = false; g.b_kfast = true;
  g.tag = "gemm_f64:small";
  GB_TRY(gemm_f64(g, s));
  if (noptorb < N || P < N) {
    GB_LAUNCH("zero_outside", s,
              zero_outside_kernel<<<cdiv((long long)N * N, 256), 256, 0, s>>>(elag, N, noptorb, P));
  }
  return GB_OK;
}

// ---------------------------------------------------------------------------
// A7  computeE_elec:  E = tr(elag[:P, :P]) + sum_i w_i C_i^T H C_i
// ---------------------------------------------------------------------------
extern "C" size_t gb_energy_elec_workspace_f64(int nbf, int nbf5) {
  Sizer z;
  z.add<double>((size_t)nbf * nbf5);
  z.add<double>((size_t)nbf5);
  return z.used;
}

extern "C" int gb_energy_elec_f64(const double* elag, const double* C, const double* H, const double* n, int nbf,
                                  int nbf5, int nbeta, int nalpha, int high_spin, double* E, void* workspace,
                                  size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5;
  GB_REQUIRE(N > 0 && P > 0 && P <= N && 0 <= nbeta && nbeta <= nalpha && nalpha <= P, GB_ERR_BAD_SHAPE,
             "gb_energy_elec_f64: bad sizes");
  GB_REQUIRE(elag && C && H && n && E, GB_ERR_INVALID_ARG, "gb_energy_elec_f64: null pointer");
  Carve cv(workspace, workspace_bytes);
  double* X = cv.take<double>((size_t)N * P);
  double* Hd = cv.take<double>((size_t)P);
  GB_REQUIRE(X && Hd, GB_ERR_WORKSPACE, "gb_energy_elec_f64: workspace too small");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GemmF64 g{};
  g.M = N; g.N = P; g.K = N; g.batch = 1;
  g.A = {H, 0, lin(N), lin(1)};
  g.B = {C, 0, lin(N), lin(1)};
  g.C = {X, 0, lin(P), lin(1)};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_NONE;
  g.a_kfast = true; g.b_kfast = false;
  g.tag = "gemm_f64:small";
  GB_TRY(gemm_f64(g, s));
  GB_TRY(launch_col_dot(C, N, X, P, Hd, N, P, s));
  GB_LAUNCH("energy_elec", s,
            energy_elec_kernel<<<1, 256, 0, s>>>(elag, Hd, n, N, P, nbeta, nalpha, high_spin, E));
  return GB_OK;
}
