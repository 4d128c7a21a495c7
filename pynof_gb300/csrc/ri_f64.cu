// Plain FP64 RI path: computeJKj (JKj_RI), computeJKH_MO (JKH_MO_RI),
// Integrals_MO_RI and computeLagrange2 (RI, closed shell).
//
// Sizes: N = nbf, P = nbf5, Q = naux.  All matrices are row-major (numpy
// C order) device arrays: C[m * N + p], b[(m * N + n) * Q + l],
// J/K[(q * N + m) * N + n], bMO[(a * P + q) * Q + l].
#include "gemm_f64.cuh"
#include "ri_kernels.cuh"

using namespace gb;

namespace {

// T[q][n][l] = sum_m C[m][q] b[m][n][l]   (the first half-transform)
int half_transform_first(const double* C, const double* b, int N, int P, int Q, double* T,
                         cudaStream_t s) {
  GemmF64 g{};
  g.M = P; g.N = N * Q; g.K = N; g.batch = 1;
  g.A = {C, 0, lin(1), lin(N)};
  g.B = {b, 0, lin((long long)N * Q), lin(1)};
  g.C = {T, 0, lin((long long)N * Q), lin(1)};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_NONE;
  g.a_kfast = false; g.b_kfast = false;
  g.tag = "gemm_f64:half_transform";
  return gemm_f64(g, s);
}

// T[q][m][l] = sum_n C[n][q] b[m][n][l]   (contracts b's second index; batch over m)
int half_transform_second(const double* C, const double* b, int N, int P, int Q, double* T,
                          cudaStream_t s) {
  GemmF64 g{};
  g.M = P; g.N = Q; g.K = N; g.batch = N;
  g.A = {C, 0, lin(1), lin(N)};
  g.B = {b, (long long)N * Q, lin(Q), lin(1)};
  g.C = {T, Q, lin((long long)N * Q), lin(1)};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_NONE;
  g.a_kfast = false; g.b_kfast = false;
  g.tag = "gemm_f64:half_transform2";
  return gemm_f64(g, s);
}

// X[m][p] = sum_n H[m][n] C[n][p]  (N x P)
int h_times_cp(const double* H, const double* C, int N, int P, double* X, cudaStream_t s) {
  GemmF64 g{};
  g.M = N; g.N = P; g.K = N; g.batch = 1;
  g.A = {H, 0, lin(N), lin(1)};
  g.B = {C, 0, lin(N), lin(1)};
  g.C = {X, 0, lin(P), lin(1)};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_NONE;
  g.a_kfast = true; g.b_kfast = false;
  g.tag = "gemm_f64:small";
  return gemm_f64(g, s);
}

int check_sizes(int N, int P, int Q) {
  GB_REQUIRE(N > 0 && P > 0 && Q > 0 && P <= N, GB_ERR_BAD_SHAPE,
             "invalid sizes nbf=%d nbf5=%d naux=%d (need 0 < nbf5 <= nbf, naux > 0)", N, P, Q);
  GB_REQUIRE(P <= 65535, GB_ERR_BAD_SHAPE, "nbf5=%d exceeds 65535", P);
  return GB_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// A1  computeJKj, RI
// ---------------------------------------------------------------------------
static void jkj_ri_layout(Sizer& z, int N, int P, int Q) {
  z.add<double>((size_t)P * N * Q);  // T
  z.add<double>((size_t)P * Q);      // d
}

extern "C" size_t gb_jkj_ri_workspace_f64(int nbf, int nbf5, int naux) {
  Sizer z;
  jkj_ri_layout(z, nbf, nbf5, naux);
  return z.used;
}

extern "C" int gb_jkj_ri_f64(const double* C, const double* b, int nbf, int nbf5, int naux, double* J,
                             double* K, void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5, Q = naux;
  GB_TRY(check_sizes(N, P, Q));
  GB_REQUIRE(C && b && J && K, GB_ERR_INVALID_ARG, "gb_jkj_ri_f64: null pointer");
  Carve cv(workspace, workspace_bytes);
  double* T = cv.take<double>((size_t)P * N * Q);
  double* d = cv.take<double>((size_t)P * Q);
  GB_REQUIRE(T && d, GB_ERR_WORKSPACE, "gb_jkj_ri_f64: workspace too small (%zu < %zu)", workspace_bytes,
             gb_jkj_ri_workspace_f64(N, P, Q));
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  GB_TRY(half_transform_first(C, b, N, P, Q, T, s));
  GB_TRY(launch_contract_diag(C, T, d, N, P, Q, s));

  // J[q][mn] = sum_l d[q][l] b[mn][l]: only pairs with n >= m are computed
  GemmF64 gj{};
  gj.M = P; gj.N = N * N; gj.K = Q; gj.batch = 1;
  gj.A = {d, 0, lin(Q), lin(1)};
  gj.B = {b, 0, lin(1), lin(Q)};
  gj.C = {J, 0, lin((long long)N * N), lin(1)};
  gj.alpha = 1.0; gj.beta = 0.0; gj.sym = SYM_PAIRCOL; gj.pair_n = N;
  gj.a_kfast = true; gj.b_kfast = true;
  gj.tag = "gemm_f64:J";
  GB_TRY(gemm_f64(gj, s));

  // K[q] = T_q T_q^T (batched SYRK, lower tiles skipped and mirrored)
  GemmF64 gk{};
  gk.M = N; gk.N = N; gk.K = Q; gk.batch = P;
  gk.A = {T, (long long)N * Q, lin(Q), lin(1)};
  gk.B = {T, (long long)N * Q, lin(1), lin(Q)};
  gk.C = {K, (long long)N * N, lin(N), lin(1)};
  gk.alpha = 1.0; gk.beta = 0.0; gk.sym = SYM_ROWCOL;
  gk.a_kfast = true; gk.b_kfast = true;
  gk.tag = "gemm_f64:K";
  GB_TRY(gemm_f64(gk, s));
  return GB_OK;
}

// ---------------------------------------------------------------------------
// A3  computeJKH_MO, RI
// ---------------------------------------------------------------------------
static void jkh_mo_ri_layout(Sizer& z, int N, int P, int Q) {
  z.add<double>((size_t)P * N * Q);  // T
  z.add<double>((size_t)P * P * Q);  // bpq
  z.add<double>((size_t)P * Q);      // d
  z.add<double>((size_t)N * P);      // X = H Cp
}

extern "C" size_t gb_jkh_mo_ri_workspace_f64(int nbf, int nbf5, int naux) {
  Sizer z;
  jkh_mo_ri_layout(z, nbf, nbf5, naux);
  return z.used;
}

extern "C" int gb_jkh_mo_ri_f64(const double* C, const double* H, const double* b, int nbf, int nbf5,
                                int naux, double* J_MO, double* K_MO, double* H_core, void* workspace,
                                size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5, Q = naux;
  GB_TRY(check_sizes(N, P, Q));
  GB_REQUIRE(C && H && b && J_MO && K_MO && H_core, GB_ERR_INVALID_ARG, "gb_jkh_mo_ri_f64: null pointer");
  Carve cv(workspace, workspace_bytes);
  double* T = cv.take<double>((size_t)P * N * Q);
  double* bpq = cv.take<double>((size_t)P * P * Q);
  double* d = cv.take<double>((size_t)P * Q);
  double* X = cv.take<double>((size_t)N * P);
  GB_REQUIRE(T && bpq && d && X, GB_ERR_WORKSPACE, "gb_jkh_mo_ri_f64: workspace too small (%zu < %zu)",
             workspace_bytes, gb_jkh_mo_ri_workspace_f64(N, P, Q));
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  GB_TRY(half_transform_first(C, b, N, P, Q, T, s));
  // bpq[p][q][l] = sum_n C[n][q] T[p][n][l]
  GemmF64 g{};
  g.M = P; g.N = Q; g.K = N; g.batch = P;
  g.A = {C, 0, lin(1), lin(N)};
  g.B = {T, (long long)N * Q, lin(Q), lin(1)};
  g.C = {bpq, (long long)P * Q, lin(Q), lin(1)};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_NONE;
  g.a_kfast = false; g.b_kfast = false;
  g.tag = "gemm_f64:bpq";
  GB_TRY(gemm_f64(g, s));

  GB_TRY(launch_gather_diag(bpq, d, P, Q, (long long)P * Q + Q, s));
  // J_MO = d d^T
  GemmF64 gj{};
  gj.M = P; gj.N = P; gj.K = Q; gj.batch = 1;
  gj.A = {d, 0, lin(Q), lin(1)};
  gj.B = {d, 0, lin(1), lin(Q)};
  gj.C = {J_MO, 0, lin(P), lin(1)};
  gj.alpha = 1.0; gj.beta = 0.0; gj.sym = SYM_ROWCOL;
  gj.a_kfast = true; gj.b_kfast = true;
  gj.tag = "gemm_f64:small";
  GB_TRY(gemm_f64(gj, s));
  GB_TRY(launch_row_sumsq(bpq, K_MO, (long long)P * P, Q, s));

  GB_TRY(h_times_cp(H, C, N, P, X, s));
  GB_TRY(launch_col_dot(C, N, X, P, H_core, N, P, s));
  return GB_OK;
}

// ---------------------------------------------------------------------------
// A5  Integrals_MO_RI:  Hmat (N x P) and bMO (N, P, Q)
// ---------------------------------------------------------------------------
static int mo_ri_core(const double* C, const double* H, const double* b, int N, int P, int Q, double* Hmat,
                      double* bMO, double* T, double* X, cudaStream_t s) {
  GB_TRY(half_transform_second(C, b, N, P, Q, T, s));
  // bMO[a][q][l] = sum_m C[m][a] T[q][m][l]   (batch q)
  GemmF64 g{};
  g.M = N; g.N = Q; g.K = N; g.batch = P;
  g.A = {C, 0, lin(1), lin(N)};
  g.B = {T, (long long)N * Q, lin(Q), lin(1)};
  g.C = {bMO, Q, lin((long long)P * Q), lin(1)};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_NONE;
  g.a_kfast = false; g.b_kfast = false;
  g.tag = "gemm_f64:bMO";
  GB_TRY(gemm_f64(g, s));
  // Hmat = C^T (H Cp)
  GB_TRY(h_times_cp(H, C, N, P, X, s));
  GemmF64 gh{};
  gh.M = N; gh.N = P; gh.K = N; gh.batch = 1;
  gh.A = {C, 0, lin(1), lin(N)};
  gh.B = {X, 0, lin(P), lin(1)};
  gh.C = {Hmat, 0, lin(P), lin(1)};
  gh.alpha = 1.0; gh.beta = 0.0; gh.sym = SYM_NONE;
  gh.a_kfast = false; gh.b_kfast = false;
  gh.tag = "gemm_f64:small";
  return gemm_f64(gh, s);
}

static void mo_ri_layout(Sizer& z, int N, int P, int Q) {
  z.add<double>((size_t)P * N * Q);  // T (second-index half transform)
  z.add<double>((size_t)N * P);      // X
}

extern "C" size_t gb_mo_ri_workspace_f64(int nbf, int nbf5, int naux) {
  Sizer z;
  mo_ri_layout(z, nbf, nbf5, naux);
  return z.used;
}

extern "C" int gb_mo_ri_f64(const double* C, const double* H, const double* b, int nbf, int nbf5, int naux,
                            double* Hmat, double* bMO, void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5, Q = naux;
  GB_TRY(check_sizes(N, P, Q));
  GB_REQUIRE(C && H && b && Hmat && bMO, GB_ERR_INVALID_ARG, "gb_mo_ri_f64: null pointer");
  Carve cv(workspace, workspace_bytes);
  double* T = cv.take<double>((size_t)P * N * Q);
  double* X = cv.take<double>((size_t)N * P);
  GB_REQUIRE(T && X, GB_ERR_WORKSPACE, "gb_mo_ri_f64: workspace too small (%zu < %zu)", workspace_bytes,
             gb_mo_ri_workspace_f64(N, P, Q));
  return mo_ri_core(C, H, b, N, P, Q, Hmat, bMO, T, X, static_cast<cudaStream_t>(stream));
}

// ---------------------------------------------------------------------------
// A5  computeLagrange2, RI, closed shell
// ---------------------------------------------------------------------------
static void lagrange2_ri_layout(Sizer& z, int N, int P, int Q) {
  z.add<double>((size_t)P * N * Q);  // T, later reused for Y (P*P*Q <= P*N*Q)
  z.add<double>((size_t)N * P * Q);  // bMO
  z.add<double>((size_t)N * P);      // X
  z.add<double>((size_t)P * Q);      // d
  z.add<double>((size_t)P * Q);      // w
  z.add<double>((size_t)P * P);      // cj12 with zero diagonal
}

extern "C" size_t gb_lagrange2_ri_workspace_f64(int nbf, int nbf5, int naux) {
  Sizer z;
  lagrange2_ri_layout(z, nbf, nbf5, naux);
  return z.used;
}

extern "C" int gb_lagrange2_ri_f64(const double* C, const double* H, const double* b, const double* n,
                                   const double* cj12, const double* ck12, int nbf, int nbf5, int naux,
                                   int nbeta, int nalpha, double* elag, double* Hmat, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5, Q = naux;
  GB_TRY(check_sizes(N, P, Q));
  GB_REQUIRE(C && H && b && n && cj12 && ck12 && elag && Hmat, GB_ERR_INVALID_ARG,
             "gb_lagrange2_ri_f64: null pointer");
  GB_REQUIRE(0 <= nbeta && nbeta <= nalpha && nalpha <= P, GB_ERR_BAD_SHAPE,
             "gb_lagrange2_ri_f64: need 0 <= nbeta <= nalpha <= nbf5");
  Carve cv(workspace, workspace_bytes);
  double* T = cv.take<double>((size_t)P * N * Q);
  double* bMO = cv.take<double>((size_t)N * P * Q);
  double* X = cv.take<double>((size_t)N * P);
  double* d = cv.take<double>((size_t)P * Q);
  double* w = cv.take<double>((size_t)P * Q);
  double* cjm = cv.take<double>((size_t)P * P);
  GB_REQUIRE(T && bMO && X && d && w && cjm, GB_ERR_WORKSPACE,
             "gb_lagrange2_ri_f64: workspace too small (%zu < %zu)", workspace_bytes,
             gb_lagrange2_ri_workspace_f64(N, P, Q));
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  GB_TRY(mo_ri_core(C, H, b, N, P, Q, Hmat, bMO, T, X, s));
  // d[b][k] = bMO[b][b][k]
  GB_TRY(launch_gather_diag(bMO, d, P, Q, (long long)P * Q + Q, s));
  // w = cj12' d + coef_b d   (cj12' has a zero diagonal; coef_b = n_b for b in doc or vir)
  GB_TRY(launch_copy_zero_diag(cj12, cjm, P, s));
  GemmF64 gw{};
  gw.M = P; gw.N = Q; gw.K = P; gw.batch = 1;
  gw.A = {cjm, 0, lin(P), lin(1)};
  gw.B = {d, 0, lin(Q), lin(1)};
  gw.C = {w, 0, lin(Q), lin(1)};
  gw.alpha = 1.0; gw.beta = 0.0; gw.sym = SYM_NONE;
  gw.a_kfast = true; gw.b_kfast = false;
  gw.tag = "gemm_f64:small";
  GB_TRY(gemm_f64(gw, s));
  GB_TRY(launch_add_scaled_rows(w, d, n, P, Q, nbeta, nalpha, s));
  // Y[b][q][k] = ck12[b][q] (q != b) bMO[b][q][k], stored over T
  double* Y = T;
  GB_TRY(launch_make_ck_weighted(bMO, ck12, Y, P, Q, s));
  // elag[a][b] = -sum_{qk} bMO[a][qk] Y[b][qk]    (b < P)
  GemmF64 ge{};
  ge.M = N; ge.N = P; ge.K = P * Q; ge.batch = 1;
  ge.A = {bMO, 0, lin((long long)P * Q), lin(1)};
  ge.B = {Y, 0, lin(1), lin((long long)P * Q)};
  ge.C = {elag, 0, lin(N), lin(1)};
  ge.alpha = -1.0; ge.beta = 0.0; ge.sym = SYM_NONE;
  ge.a_kfast = true; ge.b_kfast = true;
  ge.tag = "gemm_f64:ck_exchange";
  GB_TRY(gemm_f64(ge, s));
  // elag[a][b] += n_b Hmat[a][b] + sum_k bMO[a][b][k] w[b][k];  elag[:, P:] = 0
  GB_TRY(launch_lagrange2_finish(bMO, w, Hmat, n, elag, N, P, Q, s));
  return GB_OK;
}

// ---------------------------------------------------------------------------
// b_mnl = sum_k (mn|k) M[k][l]  (compute_integrals, integrals.py:35-49: the
// einsum "mnk,kl->mnl" with M = metric^(-1/2)); M symmetric.  (mn|k) is
// symmetric in (m, n), so only the rows m <= n are computed and mirrored.
// ---------------------------------------------------------------------------
extern "C" int gb_ri_factor_f64(const double* mnk, const double* M, int nbf, int naux, double* b, void* stream) {
  clear_error();
  const int N = nbf, Q = naux;
  GB_REQUIRE(N > 0 && Q > 0, GB_ERR_BAD_SHAPE, "gb_ri_factor_f64: bad sizes nbf=%d naux=%d", N, Q);
  GB_REQUIRE((long long)N * N <= 2147483647LL, GB_ERR_BAD_SHAPE, "gb_ri_factor_f64: nbf=%d too large", N);
  GB_REQUIRE(mnk && M && b, GB_ERR_INVALID_ARG, "gb_ri_factor_f64: null pointer");
  GemmF64 g{};
  g.M = N * N; g.N = Q; g.K = Q; g.batch = 1;
  g.A = {mnk, 0, lin(Q), lin(1)};  // A((m,n), k) = mnk[(m,n)][k]
  g.B = {M, 0, lin(Q), lin(1)};    // B(k, l) = M[k][l]
  g.C = {b, 0, lin(Q), lin(1)};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_NONE;
  g.a_kfast = true; g.b_kfast = false;
  g.tag = "gemm_f64:ri_factor";
  return gemm_f64(g, static_cast<cudaStream_t>(stream));
}

// ---------------------------------------------------------------------------
// Plain FP64 GEMM C = A B^T (row-major A [M][K], B [N][K], C [M][N]) on the
// DMMA engine, the FP64 counterpart of gb_dgemm_mixed.
// ---------------------------------------------------------------------------
extern "C" int gb_dgemm_f64(const double* A, const double* B, int M, int N, int K, double* C, void* stream) {
  clear_error();
  GB_REQUIRE(M > 0 && N > 0 && K > 0, GB_ERR_BAD_SHAPE, "gb_dgemm_f64: bad sizes M=%d N=%d K=%d", M, N, K);
  GB_REQUIRE(A && B && C, GB_ERR_INVALID_ARG, "gb_dgemm_f64: null pointer");
  GemmF64 g{};
  g.M = M; g.N = N; g.K = K; g.batch = 1;
  g.A = {A, 0, lin(K), lin(1)};
  g.B = {B, 0, lin(1), lin(K)};  // B(k, j) = B[j][k]
  g.C = {C, 0, lin(N), lin(1)};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_NONE;
  g.a_kfast = true; g.b_kfast = true;
  g.tag = "gemm_f64:dgemm";
  return gemm_f64(g, static_cast<cudaStream_t>(stream));
}

