// Plain FP64 full-ERI path: computeJKj (JKj_Full), computeJKH_MO (JKH_MO_Full),
// Integrals_MO_Full and computeLagrange2 (full ERI, closed shell).
//
// I[m][n][s][l] = (mn|sl) is the row-major N^4 tensor of the reference
// (8-fold symmetric).  D_i[s][l] = C[s][i] C[l][i].
//   J_i[(m,n)] = sum_(s,l) D_i[(s,l)] I[(m,n)][(s,l)]          (GEMM, K = N^2)
//   K_i[(m,s)] = sum_(n,l) D_i[(n,l)] I[m][n][s][l]             (GEMM whose B operand
//                 is read through the split maps (n,l) -> n N^2 + l, (m,s) -> m N^3 + s N)
// Both J_i and K_i are symmetric, so only pairs n >= m are computed (mirrored).
#include "gemm_f64.cuh"
#include "ri_kernels.cuh"

using namespace gb;

namespace {

__global__ void density_kernel(const double* __restrict__ C, double* __restrict__ D, int N, int P) {
  const long long sl = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (sl >= (long long)N * N) return;
  const int s = (int)(sl / N), l = (int)(sl % N);
  D[(long long)i * N * N + sl] = C[(long long)s * N + i] * C[(long long)l * N + i];
}

// elag[a][b] (b < P) = n_b Hmat[a][b] + c_b n_b I_MO[a,b,b,b]
//   + sum_{q != b} cj[b,q] I_MO[a,b,q,q] - sum_{q != b} ck[b,q] I_MO[a,q,b,q];  one warp per (a, b)
__global__ void lagrange2_full_kernel(const double* __restrict__ imo, const double* __restrict__ Hmat,
                                      const double* __restrict__ n, const double* __restrict__ cj,
                                      const double* __restrict__ ck, double* __restrict__ elag, int N, int P,
                                      int nbeta, int nalpha) {
  const long long w = (long long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= (long long)N * P) return;
  const int a = (int)(w / P), b = (int)(w % P);
  const long long P2 = (long long)P * P, P3 = P2 * P;
  const double* ia = imo + (long long)a * P3;
  double acc = 0.0;
  for (int q = lane; q < P; q += 32) {
    if (q == b) continue;
    acc = fma(cj[(long long)b * P + q], ia[(long long)b * P2 + (long long)q * P + q], acc);
    acc = fma(-ck[(long long)b * P + q], ia[(long long)q * P2 + (long long)b * P + q], acc);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) {
    double v = acc + n[b] * Hmat[(long long)a * P + b];
    if (b < nbeta || b >= nalpha) v += n[b] * ia[(long long)b * P2 + (long long)b * P + b];
    elag[(long long)a * N + b] = v;
  }
}

__global__ void zero_cols_from_kernel(double* __restrict__ elag, int N, int P) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int W = N - P;
  if (idx >= (long long)N * W) return;
  elag[(idx / W) * N + P + (idx % W)] = 0.0;
}

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

int check_full(int N, int P) {
  GB_REQUIRE(N > 0 && P > 0 && P <= N, GB_ERR_BAD_SHAPE, "invalid sizes nbf=%d nbf5=%d", N, P);
  GB_REQUIRE((long long)N * N <= 2147483647LL / 2, GB_ERR_BAD_SHAPE, "nbf=%d too large for the full-ERI path", N);
  return GB_OK;
}

int make_density(const double* C, double* D, int N, int P, cudaStream_t s) {
  GB_LAUNCH("density", s, density_kernel<<<dim3(cdiv((long long)N * N, 256), P), 256, 0, s>>>(C, D, N, P));
  return GB_OK;
}

int jk_full_core(const double* D, const double* I, int N, int P, double* J, double* K, cudaStream_t s) {
  const long long NN = (long long)N * N;
  GemmF64 g{};
  g.M = P; g.N = (int)NN; g.K = (int)NN; g.batch = 1;
  g.A = {D, 0, lin(NN), lin(1)};
  g.B = {I, 0, lin(1), lin(NN)};                 // B((s,l), (m,n)) = I[(m,n)][(s,l)]
  g.C = {J, 0, lin(NN), lin(1)};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_PAIRCOL; g.pair_n = N;
  g.a_kfast = true; g.b_kfast = true;
  g.tag = "gemm_f64:J_full";
  GB_TRY(gemm_f64(g, s));
  g.B = {I, 0, split(N, NN, 1), split(N, NN * N, N)};  // B((n,l), (m,s)) = I[m][n][s][l]
  g.C = {K, 0, lin(NN), lin(1)};
  g.tag = "gemm_f64:K_full";
  return gemm_f64(g, s);
}

}  // namespace

// ---------------------------------------------------------------------------
// A2  computeJKj, full ERI
// ---------------------------------------------------------------------------
extern "C" size_t gb_jkj_full_workspace_f64(int nbf, int nbf5) {
  Sizer z;
  z.add<double>((size_t)nbf5 * nbf * nbf);
  return z.used;
}

extern "C" int gb_jkj_full_f64(const double* C, const double* I, int nbf, int nbf5, double* J, double* K,
                               void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5;
  GB_TRY(check_full(N, P));
  GB_REQUIRE(C && I && J && K, GB_ERR_INVALID_ARG, "gb_jkj_full_f64: null pointer");
  Carve cv(workspace, workspace_bytes);
  double* D = cv.take<double>((size_t)P * N * N);
  GB_REQUIRE(D, GB_ERR_WORKSPACE, "gb_jkj_full_f64: workspace too small");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GB_TRY(make_density(C, D, N, P, s));
  return jk_full_core(D, I, N, P, J, K, s);
}

// ---------------------------------------------------------------------------
// A4  computeJKH_MO, full ERI:  J_MO = J D^T, K_MO = K D^T, H_core
// ---------------------------------------------------------------------------
extern "C" size_t gb_jkh_mo_full_workspace_f64(int nbf, int nbf5) {
  Sizer z;
  z.add<double>((size_t)nbf5 * nbf * nbf);  // D
  z.add<double>((size_t)nbf5 * nbf * nbf);  // J
  z.add<double>((size_t)nbf5 * nbf * nbf);  // K
  z.add<double>((size_t)nbf * nbf5);        // H C_p
  return z.used;
}

extern "C" int gb_jkh_mo_full_f64(const double* C, const double* H, const double* I, int nbf, int nbf5,
                                  double* J_MO, double* K_MO, double* H_core, void* workspace, size_t workspace_bytes,
                                  void* stream) {
  clear_error();
  const int N = nbf, P = nbf5;
  GB_TRY(check_full(N, P));
  GB_REQUIRE(C && H && I && J_MO && K_MO && H_core, GB_ERR_INVALID_ARG, "gb_jkh_mo_full_f64: null pointer");
  Carve cv(workspace, workspace_bytes);
  const size_t PNN = (size_t)P * N * N;
  double* D = cv.take<double>(PNN);
  double* J = cv.take<double>(PNN);
  double* K = cv.take<double>(PNN);
  double* X = cv.take<double>((size_t)N * P);
  GB_REQUIRE(D && J && K && X, GB_ERR_WORKSPACE, "gb_jkh_mo_full_f64: workspace too small");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GB_TRY(make_density(C, D, N, P, s));
  GB_TRY(jk_full_core(D, I, N, P, J, K, s));
  const long long NN = (long long)N * N;
  GemmF64 g{};
  g.M = P; g.N = P; g.K = (int)NN; g.batch = 1;
  g.A = {J, 0, lin(NN), lin(1)};
  g.B = {D, 0, lin(1), lin(NN)};
  g.C = {J_MO, 0, lin(P), lin(1)};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_ROWCOL;
  g.a_kfast = true; g.b_kfast = true;
  g.tag = "gemm_f64:small";
  GB_TRY(gemm_f64(g, s));
  g.A = {K, 0, lin(NN), lin(1)};
  g.C = {K_MO, 0, lin(P), lin(1)};
  GB_TRY(gemm_f64(g, s));
  // H_core[p] = C_p^T H C_p
  GemmF64 gh{};
  gh.M = N; gh.N = P; gh.K = N; gh.batch = 1;
  gh.A = {H, 0, lin(N), lin(1)};
  gh.B = {C, 0, lin(N), lin(1)};
  gh.C = {X, 0, lin(P), lin(1)};
  gh.alpha = 1.0; gh.beta = 0.0; gh.sym = SYM_NONE;
  gh.a_kfast = true; gh.b_kfast = false;
  gh.tag = "gemm_f64:small";
  GB_TRY(gemm_f64(gh, s));
  return launch_col_dot(C, N, X, P, H_core, N, P, s);
}

// ---------------------------------------------------------------------------
// A6  Integrals_MO_Full: Hmat (N x P) and I_MO[p][q][r][t] (p < N; q, r, t < P)
//     by four quarter transforms (t, then r, then q, then p).
// ---------------------------------------------------------------------------
extern "C" size_t gb_mo_full_workspace_f64(int nbf, int nbf5) {
  Sizer z;
  const size_t N = nbf, P = nbf5;
  z.add<double>(N * N * N * P);  // X1 [m][n][s][t], later X3 [m][q][r][t]
  z.add<double>(N * N * P * P);  // X2 [m][n][r][t]
  z.add<double>(N * P);          // H C_p
  return z.used;
}

static int mo_full_core(const double* C, const double* H, const double* I, int N, int P, double* Hmat,
                        double* imo, double* X1, double* X2, double* X, cudaStream_t s) {
  const long long NP = (long long)N * P, P2 = (long long)P * P, P3 = P2 * P, NN = (long long)N * N;
  GemmF64 g{};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_NONE;
  // X1[m][(n,s)][t] = sum_l I[m][(n,s)][l] C[l][t]          (batch m)
  g.M = (int)NN; g.N = P; g.K = N; g.batch = N;
  g.A = {I, NN * N, lin(N), lin(1)};
  g.B = {C, 0, lin(N), lin(1)};
  g.C = {X1, NN * P, lin(P), lin(1)};
  g.a_kfast = true; g.b_kfast = false;
  g.tag = "gemm_f64:quarter";
  GB_TRY(gemm_f64(g, s));
  // X2[(m,n)][r][t] = sum_s C[s][r] X1[(m,n)][s][t]   columns j = (mn, t)
  g.M = P; g.N = (int)(NN * P); g.K = N; g.batch = 1;
  g.A = {C, 0, lin(1), lin(N)};
  g.B = {X1, 0, lin(P), split(P, NP, 1)};
  g.C = {X2, 0, lin(P), split(P, P2, 1)};
  g.a_kfast = false; g.b_kfast = false;
  GB_TRY(gemm_f64(g, s));
  // X3[m][q][(r,t)] = sum_n C[n][q] X2[m][n][(r,t)]    columns j = (m, rt); stored over X1
  double* X3 = X1;
  g.M = P; g.N = (int)(N * P2); g.K = N; g.batch = 1;
  g.A = {C, 0, lin(1), lin(N)};
  g.B = {X2, 0, lin(P2), split(P2, N * P2, 1)};
  g.C = {X3, 0, lin(P2), split(P2, P3, 1)};
  GB_TRY(gemm_f64(g, s));
  // I_MO[p][(q,r,t)] = sum_m C[m][p] X3[m][(q,r,t)]
  g.M = N; g.N = (int)P3; g.K = N; g.batch = 1;
  g.A = {C, 0, lin(1), lin(N)};
  g.B = {X3, 0, lin(P3), lin(1)};
  g.C = {imo, 0, lin(P3), lin(1)};
  GB_TRY(gemm_f64(g, s));
  // Hmat = C^T (H C_p)
  GemmF64 gh{};
  gh.M = N; gh.N = P; gh.K = N; gh.batch = 1;
  gh.A = {H, 0, lin(N), lin(1)};
  gh.B = {C, 0, lin(N), lin(1)};
  gh.C = {X, 0, lin(P), lin(1)};
  gh.alpha = 1.0; gh.beta = 0.0; gh.sym = SYM_NONE;
  gh.a_kfast = true; gh.b_kfast = false;
  gh.tag = "gemm_f64:small";
  GB_TRY(gemm_f64(gh, s));
  gh.A = {C, 0, lin(1), lin(N)};
  gh.B = {X, 0, lin(P), lin(1)};
  gh.C = {Hmat, 0, lin(P), lin(1)};
  gh.a_kfast = false; gh.b_kfast = false;
  return gemm_f64(gh, s);
}

extern "C" int gb_mo_full_f64(const double* C, const double* H, const double* I, int nbf, int nbf5, double* Hmat,
                              double* I_MO, void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5;
  GB_TRY(check_full(N, P));
  GB_REQUIRE((long long)N * P * P * P <= 2147483647LL && (long long)N * N * P * P <= 2147483647LL * 8,
             GB_ERR_BAD_SHAPE, "gb_mo_full_f64: sizes too large");
  GB_REQUIRE(C && H && I && Hmat && I_MO, GB_ERR_INVALID_ARG, "gb_mo_full_f64: null pointer");
  Carve cv(workspace, workspace_bytes);
  double* X1 = cv.take<double>((size_t)N * N * N * P);
  double* X2 = cv.take<double>((size_t)N * N * P * P);
  double* X = cv.take<double>((size_t)N * P);
  GB_REQUIRE(X1 && X2 && X, GB_ERR_WORKSPACE, "gb_mo_full_f64: workspace too small");
  return mo_full_core(C, H, I, N, P, Hmat, I_MO, X1, X2, X, static_cast<cudaStream_t>(stream));
}

// ---------------------------------------------------------------------------
// A6  computeLagrange2, full ERI, closed shell
// ---------------------------------------------------------------------------
extern "C" size_t gb_lagrange2_full_workspace_f64(int nbf, int nbf5) {
  Sizer z;
  const size_t N = nbf, P = nbf5;
  z.add<double>(N * N * N * P);
  z.add<double>(N * N * P * P);
  z.add<double>(N * P);
  z.add<double>(N * P * P * P);  // I_MO
  return z.used;
}

extern "C" int gb_lagrange2_full_f64(const double* C, const double* H, const double* I, const double* n,
                                     const double* cj12, const double* ck12, int nbf, int nbf5, int nbeta,
                                     int nalpha, double* elag, double* Hmat, void* workspace, size_t workspace_bytes,
                                     void* stream) {
  clear_error();
  const int N = nbf, P = nbf5;
  GB_TRY(check_full(N, P));
  GB_REQUIRE((long long)N * P * P * P <= 2147483647LL, GB_ERR_BAD_SHAPE, "gb_lagrange2_full_f64: sizes too large");
  GB_REQUIRE(0 <= nbeta && nbeta <= nalpha && nalpha <= P, GB_ERR_BAD_SHAPE,
             "gb_lagrange2_full_f64: need 0 <= nbeta <= nalpha <= nbf5");
  GB_REQUIRE(C && H && I && n && cj12 && ck12 && elag && Hmat, GB_ERR_INVALID_ARG,
             "gb_lagrange2_full_f64: null pointer");
  Carve cv(workspace, workspace_bytes);
  double* X1 = cv.take<double>((size_t)N * N * N * P);
  double* X2 = cv.take<double>((size_t)N * N * P * P);
  double* X = cv.take<double>((size_t)N * P);
  double* imo = cv.take<double>((size_t)N * P * P * P);
  GB_REQUIRE(X1 && X2 && X && imo, GB_ERR_WORKSPACE, "gb_lagrange2_full_f64: workspace too small");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GB_TRY(mo_full_core(C, H, I, N, P, Hmat, imo, X1, X2, X, s));
  GB_LAUNCH("lagrange2_full", s,
            lagrange2_full_kernel<<<cdiv((long long)N * P, 8), 256, 0, s>>>(imo, Hmat, n, cj12, ck12, elag, N, P,
                                                                           nbeta, nalpha));
  if (N > P) {
    GB_LAUNCH("zero_tail_cols", s,
              zero_cols_from_kernel<<<cdiv((long long)N * (N - P), 256), 256, 0, s>>>(elag, N, P));
  }
  return GB_OK;
}

// ---------------------------------------------------------------------------
// HF-JK helpers: computeD_HF / computeDalpha_HF and JK_HF_Full_GPU
// ---------------------------------------------------------------------------
extern "C" int gb_density_hf_f64(const double* C, int nbf, int j0, int j1, double* D, void* stream) {
  clear_error();
  const int N = nbf;
  GB_REQUIRE(N > 0 && 0 <= j0 && j0 <= j1 && j1 <= N, GB_ERR_BAD_SHAPE,
             "gb_density_hf_f64: need 0 <= j0 <= j1 <= nbf (nbf=%d j0=%d j1=%d)", N, j0, j1);
  GB_REQUIRE(C && D, GB_ERR_INVALID_ARG, "gb_density_hf_f64: null pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (j1 == j0) return cuda_status(cudaMemsetAsync(D, 0, sizeof(double) * N * N, s), "cudaMemsetAsync");
  // D[m][n] = sum_j C[m][j0 + j] C[n][j0 + j]
  GemmF64 g{};
  g.M = N; g.N = N; g.K = j1 - j0; g.batch = 1;
  g.A = {C + j0, 0, lin(N), lin(1)};
  g.B = {C + j0, 0, lin(1), lin(N)};
  g.C = {D, 0, lin(N), lin(1)};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_ROWCOL;
  g.a_kfast = true; g.b_kfast = true;
  g.tag = "gemm_f64:density";
  return gemm_f64(g, s);
}

extern "C" size_t gb_jk_hf_full_workspace_f64(int nbf) {
  (void)nbf;
  return 0;
}

extern "C" int gb_jk_hf_full_f64(const double* D, const double* I, int nbf, double* J, double* K, void* workspace,
                                 size_t workspace_bytes, void* stream) {
  (void)workspace;
  (void)workspace_bytes;
  clear_error();
  GB_TRY(check_full(nbf, 1));
  GB_REQUIRE(D && I && J && K, GB_ERR_INVALID_ARG, "gb_jk_hf_full_f64: null pointer");
  return jk_full_core(D, I, nbf, 1, J, K, static_cast<cudaStream_t>(stream));
}

// ---------------------------------------------------------------------------
// Post-NOF four-index MO transforms (compute_iajb / compute_pqrt,
// integrals.py:601-662): out[p][q][r][t] = sum_{m n s l} C[m][p0+p] C[n][q0+q]
// I[m][n][s][l] C[s][r0+r] C[l][t0+t], as four quarter transforms.
// ---------------------------------------------------------------------------
extern "C" size_t gb_mo4_full_workspace_f64(int nbf, int nq, int nr, int nt) {
  Sizer z;
  const size_t N = nbf;
  const size_t x1 = N * N * N * nt, x3 = N * (size_t)nq * nr * nt;
  z.add<double>(x1 > x3 ? x1 : x3);  // X1 [m][n][s][t], later X3 [m][q][r][t]
  z.add<double>(N * N * nr * nt);    // X2 [m][n][r][t]
  return z.used;
}

extern "C" int gb_mo4_full_f64(const double* C, const double* I, int nbf, int p0, int np, int q0, int nq, int r0,
                               int nr, int t0, int nt, double* out, void* workspace, size_t workspace_bytes,
                               void* stream) {
  clear_error();
  const int N = nbf;
  GB_TRY(check_full(N, 1));
  auto range_ok = [N](int a, int n) { return a >= 0 && n >= 0 && a + n <= N; };
  GB_REQUIRE(range_ok(p0, np) && range_ok(q0, nq) && range_ok(r0, nr) && range_ok(t0, nt), GB_ERR_BAD_SHAPE,
             "gb_mo4_full_f64: orbital ranges outside [0, nbf)");
  GB_REQUIRE((long long)N * N * N <= 2147483647LL && (long long)nq * nr * nt <= 2147483647LL &&
                 (long long)N * N * nr * nt <= 2147483647LL,
             GB_ERR_BAD_SHAPE, "gb_mo4_full_f64: sizes too large");
  GB_REQUIRE(C && I && out, GB_ERR_INVALID_ARG, "gb_mo4_full_f64: null pointer");
  GB_REQUIRE(workspace_bytes >= gb_mo4_full_workspace_f64(N, nq, nr, nt), GB_ERR_WORKSPACE,
             "gb_mo4_full_f64: workspace too small");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (np == 0 || nq == 0 || nr == 0 || nt == 0) return GB_OK;
  Carve cv(workspace, workspace_bytes);
  const size_t x1 = (size_t)N * N * N * nt, x3 = (size_t)N * nq * nr * nt;
  double* X1 = cv.take<double>(x1 > x3 ? x1 : x3);
  double* X2 = cv.take<double>((size_t)N * N * nr * nt);
  const long long NN = (long long)N * N, RT = (long long)nr * nt, QRT = (long long)nq * RT;
  GemmF64 g{};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_NONE; g.batch = 1;
  g.tag = "gemm_f64:quarter";
  // X1[(m,n,s)][t] = sum_l I[(m,n,s)][l] C[l][t0+t]
  g.M = (int)(NN * N); g.N = nt; g.K = N;
  g.A = {I, 0, lin(N), lin(1)};
  g.B = {C + t0, 0, lin(N), lin(1)};
  g.C = {X1, 0, lin(nt), lin(1)};
  g.a_kfast = true; g.b_kfast = false;
  GB_TRY(gemm_f64(g, s));
  // X2[(m,n)][r][t] = sum_s C[s][r0+r] X1[(m,n)][s][t]     columns j = ((m,n), t)
  g.M = nr; g.N = (int)(NN * nt); g.K = N;
  g.A = {C + r0, 0, lin(1), lin(N)};
  g.B = {X1, 0, lin(nt), split(nt, (long long)N * nt, 1)};
  g.C = {X2, 0, lin(nt), split(nt, RT, 1)};
  g.a_kfast = false; g.b_kfast = false;
  GB_TRY(gemm_f64(g, s));
  // X3[m][q][(r,t)] = sum_n C[n][q0+q] X2[m][n][(r,t)]     columns j = (m, (r,t)); over X1
  double* X3 = X1;
  g.M = nq; g.N = (int)(N * RT); g.K = N;
  g.A = {C + q0, 0, lin(1), lin(N)};
  g.B = {X2, 0, lin(RT), split(RT, N * RT, 1)};
  g.C = {X3, 0, lin(RT), split(RT, QRT, 1)};
  GB_TRY(gemm_f64(g, s));
  // out[p][(q,r,t)] = sum_m C[m][p0+p] X3[m][(q,r,t)]
  g.M = np; g.N = (int)QRT; g.K = N;
  g.A = {C + p0, 0, lin(1), lin(N)};
  g.B = {X3, 0, lin(QRT), lin(1)};
  g.C = {out, 0, lin(QRT), lin(1)};
  return gemm_f64(g, s);
}

