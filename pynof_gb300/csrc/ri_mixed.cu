// Split-product (tcgen05) RI path: computeJKj with FP64-accurate results from
// bf16 digit slices.  See ozaki_tc.cuh for the arithmetic.
//
// The RI factor is sliced once ("prepared") into two K-major digit copies:
//   bT[j = (n, l)][m]  (K = m, for the half transform T = C_p^T b)
//   bJ[r = (m, n), m <= n][l]  (K = l, for J = d b^T; b and J_q are symmetric
//                      in (m, n), so only the packed upper triangle of the
//                      pairs is kept and J's GEMM writes each pair twice)
// and stays resident across builds, like b itself in PyNOF's GPU path.
#include "gemm_f64.cuh"
#include "ozaki_tc.cuh"
#include "ri_kernels.cuh"
#include "slice.cuh"

using namespace gb;

namespace {

// Orbitals on the N side of the tiles (the ragged last tile is only as wide as
// it needs) when that pads less than 128-row tiles of orbitals: e.g. 300
// orbitals take 304 columns instead of 384 rows.
bool orbitals_on_n(long long P, long long rows) {
  const long long rows128 = (rows + 127) / 128 * 128;
  const long long normal = (P + 127) / 128 * 128 * rows128;
  const long long swapped = rows128 * (P / 128 * 128 + ((P % 128) + 15) / 16 * 16);
  return swapped < normal;
}

// T[q][(n,l)] = sum_m C[m][q] b[m][(n,l)] from the sliced C^T (A, rows q) and b (bT)
int half_transform_gemm(const SlicedDesc& A, const SlicedDesc& bT, int N, int P, int Q, double* Tf,
                        unsigned int* ctr, cudaStream_t s) {
  OzGemm gt{};
  gt.K = N; gt.batch = 1; gt.S = A.code(); gt.C = Tf; gt.c_sb = 0; gt.sym = SYM_NONE; gt.tag = "ozaki_tc:half_transform";
  gt.tile_counter = ctr;
  if (orbitals_on_n(P, (long long)N * Q)) {
    gt.M = N * Q; gt.N = P; gt.c_r = lin(1); gt.c_c = lin((long long)N * Q);
    return ozaki_gemm(bT, A, gt, s);
  }
  gt.M = P; gt.N = N * Q; gt.c_r = lin((long long)N * Q); gt.c_c = lin(1);
  return ozaki_gemm(A, bT, gt, s);
}

struct Prepared {
  SlicedDesc bT, bJ;
};

template <class C>
void prepared_layout(C& c, int N, int Q, int S, Prepared* out) {
  SlicedDesc t = take_sliced(c, 1, N * Q, N, S);
  SlicedDesc j = take_sliced(c, 1, N * (N + 1) / 2, Q, S);
  if (out) {
    out->bT = t;
    out->bJ = j;
  }
}


int check_mixed(int N, int P, int Q, int S) {
  GB_REQUIRE(N > 0 && P > 0 && Q > 0 && P <= N, GB_ERR_BAD_SHAPE,
             "invalid sizes nbf=%d nbf5=%d naux=%d (need 0 < nbf5 <= nbf, naux > 0)", N, P, Q);
  GB_REQUIRE(valid_split(S), GB_ERR_INVALID_ARG, "nslices=%d is neither 1..6 nor GB_SPLIT_TF32X3", S);
  GB_REQUIRE((long long)N * Q < 2147483647LL && (long long)N * N < 2147483647LL, GB_ERR_BAD_SHAPE,
             "sizes too large");
  return GB_OK;
}

struct JkjMixedWs {
  SlicedDesc A, d, T;
  double* Tf;
  double* dv;
  unsigned int* ctr;  // tile counter of the persistent GEMMs
};

template <class C>
void jkj_mixed_layout(C& c, int N, int P, int Q, int S, JkjMixedWs* w) {
  SlicedDesc A = take_sliced(c, 1, P, N, S);
  auto* tf = c.template take<double>((size_t)P * N * Q);
  auto* dv = c.template take<double>((size_t)P * Q);
  SlicedDesc d = take_sliced(c, 1, P, Q, S);
  SlicedDesc T = take_sliced(c, P, N, Q, S);
  auto* ctr = c.template take<unsigned int>(1);
  if (w) {
    w->A = A;
    w->Tf = tf;
    w->dv = dv;
    w->d = d;
    w->T = T;
    w->ctr = ctr;
  }
}


}  // namespace

extern "C" size_t gb_ri_prepare_bytes_mixed(int nbf, int naux, int nslices) {
  SizeCarve c;
  prepared_layout(c, nbf, naux, nslices, nullptr);
  return c.used;
}

extern "C" int gb_ri_prepare_mixed(const double* b, int nbf, int naux, int nslices, void* prep, size_t prep_bytes,
                                   void* stream) {
  clear_error();
  const int N = nbf, Q = naux, S = nslices;
  GB_TRY(check_mixed(N, 1, Q, S));
  GB_REQUIRE(b && prep, GB_ERR_INVALID_ARG, "gb_ri_prepare_mixed: null pointer");
  GB_REQUIRE(prep_bytes >= gb_ri_prepare_bytes_mixed(N, Q, S), GB_ERR_WORKSPACE,
             "gb_ri_prepare_mixed: buffer too small (%zu < %zu)", prep_bytes, gb_ri_prepare_bytes_mixed(N, Q, S));
  Carve c(prep, prep_bytes);
  Prepared pr;
  prepared_layout(c, N, Q, S, &pr);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // bT rows j = n*Q + l over K = m: element b[m][j]   (rows are the unit stride)
  GB_TRY(slice_operand(SliceSrc{b, 0, lin(1), lin((long long)N * Q), false}, pr.bT, s));
  // bJ rows r = (m, n), m <= n, over K = l: element b[m*N + n][l]  (K is the unit stride)
  GB_TRY(slice_operand(SliceSrc{b, 0, lin(Q), lin(1), true, N}, pr.bJ, s));
  return GB_OK;
}

extern "C" size_t gb_jkj_ri_workspace_mixed(int nbf, int nbf5, int naux, int nslices) {
  SizeCarve c;
  jkj_mixed_layout(c, nbf, nbf5, naux, nslices, nullptr);
  return c.used;
}

namespace {
// The build's prelude: slices C^T, forms T (half transform) and d, slices d.
// Leaves T, d's slices and the row exponents of T's slicing in the
// workspace for jkj_mixed_jr and jkj_mixed_k.
int jkj_mixed_t(const double* C, const Prepared& pr, const JkjMixedWs& w, int N, int P, int Q, cudaStream_t s) {
  // A rows q over K = m: element C[m][q]
  GB_TRY(slice_operand(SliceSrc{C, 0, lin(1), lin(N), false}, w.A, s));
  // T[q][(n,l)] = sum_m C[m][q] b[m][(n,l)]
  GB_TRY(half_transform_gemm(w.A, pr.bT, N, P, Q, w.Tf, w.ctr, s));
  // the contraction also records the row exponents of T's slicing (jkj_mixed_k)
  GB_TRY(launch_contract_diag(C, w.Tf, w.dv, N, P, Q, s, w.T.kind == 0 ? w.T.exps : nullptr));
  return slice_operand(SliceSrc{w.dv, 0, lin(Q), lin(1), true}, w.d, s);
}

// J[q][(m,n)] = sum_l d[q][l] b[(m,n)][l] for orbitals q0 <= q < q1 (q0 a
// multiple of the 128-row slice block, so the range starts a block of d's
// slices).  bJ's rows are the pairs m <= n; each result is also written to (n, m).
int jkj_mixed_jr(const Prepared& pr, const JkjMixedWs& w, int N, int P, int Q, int S, int q0, int q1, double* J,
                 cudaStream_t s) {
  if (q1 <= q0) return GB_OK;
  SlicedDesc d = w.d;
  d.planes = reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<unsigned char*>(w.d.planes) +
                                              (size_t)(q0 / SL_ROWS) * (size_t)w.d.kblocks() * w.d.block_bytes());
  d.exps = w.d.exps + q0;
  d.rows = q1 - q0;
  OzGemm gj{};
  gj.K = Q; gj.batch = 1; gj.S = S; gj.C = J + (size_t)q0 * N * N; gj.c_sb = 0; gj.pair_n = N; gj.tag = "ozaki_tc:J";
  gj.tile_counter = w.ctr;
  const int npairs = N * (N + 1) / 2;
  if (orbitals_on_n(P, npairs)) {
    gj.M = npairs; gj.N = q1 - q0; gj.c_r = lin(1); gj.c_c = lin((long long)N * N); gj.sym = SYM_TRIROW;
    return ozaki_gemm(pr.bJ, d, gj, s);
  }
  gj.M = q1 - q0; gj.N = npairs; gj.c_r = lin((long long)N * N); gj.c_c = lin(1); gj.sym = SYM_TRICOL;
  return ozaki_gemm(d, pr.bJ, gj, s);
}

// The J half of the build: the prelude, then J for every orbital.
int jkj_mixed_j(const double* C, const Prepared& pr, const JkjMixedWs& w, int N, int P, int Q, int S, double* J,
                cudaStream_t s) {
  GB_TRY(jkj_mixed_t(C, pr, w, N, P, Q, s));
  return jkj_mixed_jr(pr, w, N, P, Q, S, 0, P, J, s);
}

// The K half for orbitals q0 <= q < q1: K[q] = T_q T_q^T from the T that
// jkj_mixed_j left in the workspace.
int jkj_mixed_k(const JkjMixedWs& w, int N, int Q, int S, int q0, int q1, double* K, cudaStream_t s) {
  if (q1 <= q0) return GB_OK;
  SlicedDesc T = w.T;
  T.planes = reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<unsigned char*>(w.T.planes) +
                                              (size_t)q0 * (size_t)w.T.batch_bytes());
  T.exps = w.T.exps + (size_t)q0 * N;
  T.batch = q1 - q0;
  GB_TRY(slice_operand(SliceSrc{w.Tf + (size_t)q0 * N * Q, (long long)N * Q, lin(Q), lin(1), true}, T, s,
                       T.kind == 0));
  OzGemm gk{};
  gk.M = N; gk.N = N; gk.K = Q; gk.batch = q1 - q0; gk.S = S;
  // K_q is symmetric: the tile is stored transposed (rows on the unit stride),
  // which lets the epilogue store straight from its TMEM-lane layout
  gk.C = K + (size_t)q0 * N * N; gk.c_sb = (long long)N * N; gk.c_r = lin(1); gk.c_c = lin(N);
  gk.sym = SYM_ROWCOL; gk.tag = "ozaki_tc:K"; gk.tile_counter = w.ctr;
  return ozaki_gemm(T, T, gk, s);
}

int jkj_mixed_check(const char* who, int N, int P, int Q, int S, size_t workspace_bytes) {
  GB_TRY(check_mixed(N, P, Q, S));
  GB_REQUIRE(workspace_bytes >= gb_jkj_ri_workspace_mixed(N, P, Q, S), GB_ERR_WORKSPACE,
             "%s: workspace too small (%zu < %zu)", who, workspace_bytes, gb_jkj_ri_workspace_mixed(N, P, Q, S));
  return GB_OK;
}
}  // namespace

extern "C" int gb_jkj_ri_mixed(const double* C, const void* prep, int nbf, int nbf5, int naux, int nslices, double* J,
                               double* K, void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5, Q = naux, S = nslices;
  GB_TRY(jkj_mixed_check("gb_jkj_ri_mixed", N, P, Q, S, workspace_bytes));
  GB_REQUIRE(C && prep && J && K && workspace, GB_ERR_INVALID_ARG, "gb_jkj_ri_mixed: null pointer");
  Carve pc(const_cast<void*>(prep), gb_ri_prepare_bytes_mixed(N, Q, S));
  Prepared pr;
  prepared_layout(pc, N, Q, S, &pr);
  Carve wc(workspace, workspace_bytes);
  JkjMixedWs w;
  jkj_mixed_layout(wc, N, P, Q, S, &w);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GB_TRY(jkj_mixed_j(C, pr, w, N, P, Q, S, J, s));
  return jkj_mixed_k(w, N, Q, S, 0, P, K, s);
}

extern "C" int gb_jkj_ri_mixed_j(const double* C, const void* prep, int nbf, int nbf5, int naux, int nslices,
                                 double* J, void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5, Q = naux, S = nslices;
  GB_TRY(jkj_mixed_check("gb_jkj_ri_mixed_j", N, P, Q, S, workspace_bytes));
  GB_REQUIRE(C && prep && J && workspace, GB_ERR_INVALID_ARG, "gb_jkj_ri_mixed_j: null pointer");
  Carve pc(const_cast<void*>(prep), gb_ri_prepare_bytes_mixed(N, Q, S));
  Prepared pr;
  prepared_layout(pc, N, Q, S, &pr);
  Carve wc(workspace, workspace_bytes);
  JkjMixedWs w;
  jkj_mixed_layout(wc, N, P, Q, S, &w);
  return jkj_mixed_j(C, pr, w, N, P, Q, S, J, static_cast<cudaStream_t>(stream));
}

extern "C" int gb_jkj_ri_mixed_t(const double* C, const void* prep, int nbf, int nbf5, int naux, int nslices,
                                 void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5, Q = naux, S = nslices;
  GB_TRY(jkj_mixed_check("gb_jkj_ri_mixed_t", N, P, Q, S, workspace_bytes));
  GB_REQUIRE(C && prep && workspace, GB_ERR_INVALID_ARG, "gb_jkj_ri_mixed_t: null pointer");
  Carve pc(const_cast<void*>(prep), gb_ri_prepare_bytes_mixed(N, Q, S));
  Prepared pr;
  prepared_layout(pc, N, Q, S, &pr);
  Carve wc(workspace, workspace_bytes);
  JkjMixedWs w;
  jkj_mixed_layout(wc, N, P, Q, S, &w);
  return jkj_mixed_t(C, pr, w, N, P, Q, static_cast<cudaStream_t>(stream));
}

extern "C" int gb_jkj_ri_mixed_jr(const void* prep, int nbf, int nbf5, int naux, int nslices, int q0, int q1,
                                  double* J, void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5, Q = naux, S = nslices;
  GB_TRY(jkj_mixed_check("gb_jkj_ri_mixed_jr", N, P, Q, S, workspace_bytes));
  GB_REQUIRE(prep && J && workspace, GB_ERR_INVALID_ARG, "gb_jkj_ri_mixed_jr: null pointer");
  GB_REQUIRE(0 <= q0 && q0 <= q1 && q1 <= P && q0 % SL_ROWS == 0, GB_ERR_BAD_SHAPE,
             "gb_jkj_ri_mixed_jr: need 0 <= q0 <= q1 <= nbf5 and q0 a multiple of %d (%d, %d, %d)", SL_ROWS, q0, q1,
             P);
  Carve pc(const_cast<void*>(prep), gb_ri_prepare_bytes_mixed(N, Q, S));
  Prepared pr;
  prepared_layout(pc, N, Q, S, &pr);
  Carve wc(workspace, workspace_bytes);
  JkjMixedWs w;
  jkj_mixed_layout(wc, N, P, Q, S, &w);
  return jkj_mixed_jr(pr, w, N, P, Q, S, q0, q1, J, static_cast<cudaStream_t>(stream));
}

extern "C" int gb_jkj_ri_mixed_k(int nbf, int nbf5, int naux, int nslices, int q0, int q1, double* K,
                                 void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5, Q = naux, S = nslices;
  GB_TRY(jkj_mixed_check("gb_jkj_ri_mixed_k", N, P, Q, S, workspace_bytes));
  GB_REQUIRE(K && workspace, GB_ERR_INVALID_ARG, "gb_jkj_ri_mixed_k: null pointer");
  GB_REQUIRE(0 <= q0 && q0 <= q1 && q1 <= P, GB_ERR_BAD_SHAPE, "gb_jkj_ri_mixed_k: need 0 <= q0 <= q1 <= nbf5 (%d, %d, %d)",
             q0, q1, P);
  Carve wc(workspace, workspace_bytes);
  JkjMixedWs w;
  jkj_mixed_layout(wc, N, P, Q, S, &w);
  return jkj_mixed_k(w, N, Q, S, q0, q1, K, static_cast<cudaStream_t>(stream));
}

extern "C" int gb_device_status(int reset, int* status) {
  clear_error();
  GB_REQUIRE(status, GB_ERR_INVALID_ARG, "gb_device_status: null pointer");
  return ozaki_status(reset, status);
}

// ---------------------------------------------------------------------------
// Generic FP64-accurate GEMM on the tensor cores: C = A B^T (row-major A [M][K],
// B [N][K], C [M][N]).
// ---------------------------------------------------------------------------
namespace {
template <class Cv>
void dgemm_layout(Cv& c, int M, int N, int K, int S, SlicedDesc* a, SlicedDesc* b, unsigned int** ctr) {
  SlicedDesc sa = take_sliced(c, 1, M, K, S);
  SlicedDesc sb = take_sliced(c, 1, N, K, S);
  auto* ct = c.template take<unsigned int>(1);
  if (a) *a = sa;
  if (b) *b = sb;
  if (ctr) *ctr = ct;
}
}  // namespace

extern "C" size_t gb_dgemm_mixed_workspace(int M, int N, int K, int nslices) {
  SizeCarve c;
  dgemm_layout(c, M, N, K, nslices, nullptr, nullptr, nullptr);
  return c.used;
}

extern "C" int gb_dgemm_mixed(const double* A, const double* B, int M, int N, int K, int nslices, double* C,
                              void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  GB_REQUIRE(M > 0 && N > 0 && K > 0, GB_ERR_BAD_SHAPE, "gb_dgemm_mixed: bad sizes M=%d N=%d K=%d", M, N, K);
  GB_REQUIRE(valid_split(nslices), GB_ERR_INVALID_ARG, "gb_dgemm_mixed: nslices=%d is neither 1..6 nor GB_SPLIT_TF32X3",
             nslices);
  GB_REQUIRE(A && B && C, GB_ERR_INVALID_ARG, "gb_dgemm_mixed: null pointer");
  GB_REQUIRE(workspace_bytes >= gb_dgemm_mixed_workspace(M, N, K, nslices), GB_ERR_WORKSPACE,
             "gb_dgemm_mixed: workspace too small");
  Carve wc(workspace, workspace_bytes);
  SlicedDesc sa, sb;
  unsigned int* ctr = nullptr;
  dgemm_layout(wc, M, N, K, nslices, &sa, &sb, &ctr);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GB_TRY(slice_operand(SliceSrc{A, 0, lin(K), lin(1), true}, sa, s));
  GB_TRY(slice_operand(SliceSrc{B, 0, lin(K), lin(1), true}, sb, s));
  OzGemm g{};
  g.M = M; g.N = N; g.K = K; g.batch = 1; g.S = nslices;
  g.C = C; g.c_sb = 0; g.c_r = lin(N); g.c_c = lin(1);
  g.sym = SYM_NONE; g.tag = "ozaki_tc:dgemm"; g.tile_counter = ctr;
  return ozaki_gemm(sa, sb, g, s);
}

// ---------------------------------------------------------------------------
// A3  computeJKH_MO, RI, on the tensor cores
//   T  = C_p^T b                   (half transform, as in the JK build)
//   bpq[p][q][l] = sum_n C[n][q] T[p][n][l]   (batched over p; T read with K = n)
//   J_MO = d d^T (d[p] = bpq[p][p]),  K_MO[p][q] = sum_l bpq[p][q][l]^2,  H_core
// ---------------------------------------------------------------------------
namespace {
struct JkhMixedWs {
  SlicedDesc A, Tt, dS;
  double *Tf, *bpq, *d, *X;
  unsigned int* ctr;  // tile counter of the persistent GEMMs
};

template <class Cv>
void jkh_mixed_layout(Cv& c, int N, int P, int Q, int S, JkhMixedWs* w) {
  SlicedDesc A = take_sliced(c, 1, P, N, S);
  auto* tf = c.template take<double>((size_t)P * N * Q);
  SlicedDesc Tt = take_sliced(c, P, Q, N, S);
  auto* bpq = c.template take<double>((size_t)P * P * Q);
  auto* d = c.template take<double>((size_t)P * Q);
  auto* X = c.template take<double>((size_t)N * P);
  auto* ctr = c.template take<unsigned int>(1);
  SlicedDesc dS = take_sliced(c, 1, P, Q, S);  // d rows p, K = l (J_MO)
  if (w) *w = JkhMixedWs{A, Tt, dS, tf, bpq, d, X, ctr};
}

// H_core[p] = C_p^T H C_p and (optionally) Hmat = C^T H C_p in FP64
int hcore_f64(const double* C, const double* H, int N, int P, double* X, double* H_core, double* Hmat,
              cudaStream_t s) {
  GemmF64 g{};
  g.M = N; g.N = P; g.K = N; g.batch = 1;
  g.A = {H, 0, lin(N), lin(1)};
  g.B = {C, 0, lin(N), lin(1)};
  g.C = {X, 0, lin(P), lin(1)};
  g.alpha = 1.0; g.beta = 0.0; g.sym = SYM_NONE;
  g.a_kfast = true; g.b_kfast = false;
  g.tag = "gemm_f64:small";
  GB_TRY(gemm_f64(g, s));
  if (H_core) GB_TRY(launch_col_dot(C, N, X, P, H_core, N, P, s));
  if (Hmat) {
    g.A = {C, 0, lin(1), lin(N)};
    g.B = {X, 0, lin(P), lin(1)};
    g.C = {Hmat, 0, lin(P), lin(1)};
    g.a_kfast = false; g.b_kfast = false;
    GB_TRY(gemm_f64(g, s));
  }
  return GB_OK;
}

int half_transform_mixed(const double* C, const SlicedDesc& A, const SlicedDesc& bT, int N, int P, int Q,
                         double* Tf, unsigned int* ctr, cudaStream_t s) {
  GB_TRY(slice_operand(SliceSrc{C, 0, lin(1), lin(N), false}, A, s));
  return half_transform_gemm(A, bT, N, P, Q, Tf, ctr, s);
}
}  // namespace

extern "C" size_t gb_jkh_mo_ri_workspace_mixed(int nbf, int nbf5, int naux, int nslices) {
  SizeCarve c;
  jkh_mixed_layout(c, nbf, nbf5, naux, nslices, nullptr);
  return c.used;
}

extern "C" int gb_jkh_mo_ri_mixed(const double* C, const double* H, const void* prep, int nbf, int nbf5, int naux,
                                  int nslices, double* J_MO, double* K_MO, double* H_core, void* workspace,
                                  size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5, Q = naux, S = nslices;
  GB_TRY(check_mixed(N, P, Q, S));
  GB_REQUIRE(C && H && prep && J_MO && K_MO && H_core, GB_ERR_INVALID_ARG, "gb_jkh_mo_ri_mixed: null pointer");
  GB_REQUIRE(workspace_bytes >= gb_jkh_mo_ri_workspace_mixed(N, P, Q, S), GB_ERR_WORKSPACE,
             "gb_jkh_mo_ri_mixed: workspace too small");
  Carve pc(const_cast<void*>(prep), gb_ri_prepare_bytes_mixed(N, Q, S));
  Prepared pr;
  prepared_layout(pc, N, Q, S, &pr);
  Carve wc(workspace, workspace_bytes);
  JkhMixedWs w;
  jkh_mixed_layout(wc, N, P, Q, S, &w);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GB_TRY(half_transform_mixed(C, w.A, pr.bT, N, P, Q, w.Tf, w.ctr, s));
  // T read with rows l and K = n: element T[p][n][l]
  GB_TRY(slice_operand(SliceSrc{w.Tf, (long long)N * Q, lin(1), lin(Q), false}, w.Tt, s));
  OzGemm gq{};
  gq.K = N; gq.batch = P; gq.S = S; gq.C = w.bpq; gq.c_sb = (long long)P * Q; gq.sym = SYM_NONE; gq.tag = "ozaki_tc:bpq";
  gq.tile_counter = w.ctr;
  if (orbitals_on_n(P, Q)) {
    gq.M = Q; gq.N = P; gq.c_r = lin(1); gq.c_c = lin(Q);
    GB_TRY(ozaki_gemm(w.Tt, w.A, gq, s));
  } else {
    gq.M = P; gq.N = Q; gq.c_r = lin(Q); gq.c_c = lin(1);
    GB_TRY(ozaki_gemm(w.A, w.Tt, gq, s));
  }
  GB_TRY(launch_gather_diag(w.bpq, w.d, P, Q, (long long)P * Q + Q, s));
  // J_MO = d d^T (symmetric: the SYRK form, stored transposed)
  GB_TRY(slice_operand(SliceSrc{w.d, 0, lin(Q), lin(1), true}, w.dS, s));
  OzGemm gj{};
  gj.M = P; gj.N = P; gj.K = Q; gj.batch = 1; gj.S = S;
  gj.C = J_MO; gj.c_sb = 0; gj.c_r = lin(1); gj.c_c = lin(P);
  gj.sym = SYM_ROWCOL; gj.tag = "ozaki_tc:J_MO"; gj.tile_counter = w.ctr;
  GB_TRY(ozaki_gemm(w.dS, w.dS, gj, s));
  GB_TRY(launch_row_sumsq(w.bpq, K_MO, (long long)P * P, Q, s));
  return hcore_f64(C, H, N, P, w.X, H_core, nullptr, s);
}

// ---------------------------------------------------------------------------
// A5  computeLagrange2, RI, closed shell, on the tensor cores
//   bMO[a][q][l] = sum_m C[m][a] T[q][m][l]  (T[q][m][l] = sum_n C[n][q] b[m][n][l]
//   equals the half transform because b is symmetric in (m, n))
//   elag = -bMO . (ck12-weighted bMO)^T (K = nbf5 naux) + FP64 terms.
// ---------------------------------------------------------------------------
namespace {
struct Lag2MixedWs {
  SlicedDesc Ap, Tt, Sx, Sy;
  SlicedDesc dS, dT, cjS, Ct, Zt;  // the small GEMMs' operands (w, J_MO, elag = -C^T Z)
  double *Tf, *bMO, *Y, *X, *d, *w, *cjm;
  double* part;  // ns partial exchange products (ns > 1)
  double* Z;     // Z[m][b] = sum_(q,l) T[q][m][l] Y[b][q][l]
  int ns, kc;    // K splits of the exchange GEMM (whole ranges of orbitals q) and K per split
  unsigned int* ctr;  // tile counter of the persistent GEMMs
};

// K splits of the exchange GEMM (M = nbf5, N = nbf, K = nbf5 naux): with few
// output tiles the long K would run on a few CTAs, so it is cut into ranges
// of >= 768 that run as a batch; the partial products are summed in a fixed
// order (deterministic).  Each split covers whole orbitals q (nbf5 divisible
// by the split count), so its part of T is one strided block.
int exchange_splits(int N, int P, int Q) {
  const long long tiles = (long long)((N + 127) / 128) * ((P + 127) / 128);
  const long long K = (long long)P * Q;
  if (tiles >= 76 || K < 2 * 768) return 1;
  long long s = (152 + tiles - 1) / tiles;
  s = s < K / 768 ? s : K / 768;
  s = s < 64 ? s : 64;
  while (s > 1 && P % s != 0) --s;  // equal ranges of whole orbitals
  return (int)s;
}

// out[r][c] (row stride ld) = sum_s part[s][r][c], r < rows, c < cols
__global__ void sum_splits_kernel(const double* __restrict__ part, int ns, int rows, int cols,
                                  double* __restrict__ out, int ld) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)rows * cols) return;
  const long long RC = (long long)rows * cols;
  double v = 0.0;
  for (int s = 0; s < ns; ++s) v += part[s * RC + idx];
  out[(idx / cols) * ld + idx % cols] = v;
}

template <class Cv>
void lag2_mixed_layout(Cv& c, int N, int P, int Q, int S, Lag2MixedWs* w) {
  SlicedDesc Ap = take_sliced(c, 1, P, N, S);
  auto* tf = c.template take<double>((size_t)P * N * Q);
  SlicedDesc Tt = take_sliced(c, P, Q, N, S);
  auto* bmo = c.template take<double>((size_t)P * P * Q);
  auto* Y = c.template take<double>((size_t)P * P * Q);
  const int ns = exchange_splits(N, P, Q);
  const int kc = (P / ns) * Q;  // K per split: P / ns whole orbitals
  SlicedDesc Sx = take_sliced(c, ns, N, kc, S);
  SlicedDesc Sy = take_sliced(c, ns, P, kc, S);
  auto* part = ns > 1 ? c.template take<double>((size_t)ns * N * P) : nullptr;
  auto* Z = c.template take<double>((size_t)N * P);
  auto* X = c.template take<double>((size_t)N * P);
  auto* d = c.template take<double>((size_t)P * Q);
  auto* wv = c.template take<double>((size_t)P * Q);
  auto* cjm = c.template take<double>((size_t)P * P);
  auto* ctr = c.template take<unsigned int>(1);
  SlicedDesc dS = take_sliced(c, 1, P, Q, S);  // d rows p, K = l
  SlicedDesc dT = take_sliced(c, 1, Q, P, S);  // d^T rows l, K = q
  SlicedDesc cjS = take_sliced(c, 1, P, P, S);  // cj12 (zero diagonal) rows b, K = q
  SlicedDesc Ct = take_sliced(c, 1, N, N, S);  // C^T rows a, K = m
  SlicedDesc Zt = take_sliced(c, 1, P, N, S);  // Z^T rows b, K = m
  if (w) *w = Lag2MixedWs{Ap, Tt, Sx, Sy, dS, dT, cjS, Ct, Zt, tf, bmo, Y, X, d, wv, cjm, part, Z, ns, kc, ctr};
}
}  // namespace

extern "C" size_t gb_lagrange2_ri_workspace_mixed(int nbf, int nbf5, int naux, int nslices) {
  SizeCarve c;
  lag2_mixed_layout(c, nbf, nbf5, naux, nslices, nullptr);
  return c.used;
}

namespace {
// computeLagrange2 on the tensor cores; with J_MO, K_MO, H_core non-null also
// computeJKH_MO at the same orbitals, from the same transform: bMO[a][q][l] =
// (aq|l) for a, q < nbf5, so d[p] = bMO[p][p], J_MO = d d^T and
// K_MO[p][q] = sum_l bMO[p][q][l]^2, H_core[p] = C_p^T H C_p.
//
// The Lagrangian (utils.py:262-382, closed shell) is
//   elag[a][b] = n_b Hmat[a][b] + sum_k bMO[a][b][k] w[b][k]
//                - sum_(q,k) ck12[b][q] bMO[a][q][k] bMO[b][q][k]     (b < nbf5)
// for every a < nbf.  With Y[b][q][k] = ck12[b][q] bMO[b][q][k] (q != b) and
// -w[b][k] on the diagonal blocks, the last two terms are
// -sum_(q,k) bMO[a][q][k] Y[b][q][k] = -sum_m C[m][a] Z[m][b] with
// Z[m][b] = sum_(q,k) T[q][m][k] Y[b][q][k]: the MO transform is needed for
// a < nbf5 only (Y, d), and the tensor-core GEMM contracts T with Y instead.
int lagrange2_mixed_body(const double* C, const double* H, const void* prep, const double* n, const double* cj12,
                         const double* ck12, int N, int P, int Q, int nbeta, int nalpha, int S, double* elag,
                         double* Hmat, double* J_MO, double* K_MO, double* H_core, void* workspace,
                         size_t workspace_bytes, cudaStream_t s) {
  Carve pc(const_cast<void*>(prep), gb_ri_prepare_bytes_mixed(N, Q, S));
  Prepared pr;
  prepared_layout(pc, N, Q, S, &pr);
  Carve wc(workspace, workspace_bytes);
  Lag2MixedWs w;
  lag2_mixed_layout(wc, N, P, Q, S, &w);

  // C^T rows a < nbf5 (K = m): the half transform's and the MO transform's A
  GB_TRY(slice_operand(SliceSrc{C, 0, lin(1), lin(N), false}, w.Ap, s));
  GB_TRY(half_transform_gemm(w.Ap, pr.bT, N, P, Q, w.Tf, w.ctr, s));
  GB_TRY(slice_operand(SliceSrc{w.Tf, (long long)N * Q, lin(1), lin(Q), false}, w.Tt, s));
  // bMO[a][q][l], a < nbf5 (batch q): rows l (the output's unit stride, the
  // persistent form) x orbitals a on the N tile (a ragged orbital count pads
  // less there)
  OzGemm gm{};
  gm.M = Q; gm.N = P; gm.K = N; gm.batch = P; gm.S = S;
  gm.C = w.bMO; gm.c_sb = Q; gm.c_r = lin(1); gm.c_c = lin((long long)P * Q);
  gm.sym = SYM_NONE; gm.tag = "ozaki_tc:bMO"; gm.tile_counter = w.ctr;
  GB_TRY(ozaki_gemm(w.Tt, w.Ap, gm, s));
  GB_TRY(hcore_f64(C, H, N, P, w.X, H_core, Hmat, s));
  GB_TRY(launch_gather_diag(w.bMO, w.d, P, Q, (long long)P * Q + Q, s));
  // d's slices: rows p over K = l (J_MO) and rows l over K = q (w)
  GB_TRY(slice_operand(SliceSrc{w.d, 0, lin(Q), lin(1), true}, w.dS, s));
  GB_TRY(slice_operand(SliceSrc{w.d, 0, lin(1), lin(Q), false}, w.dT, s));
  if (J_MO) {
    // J_MO = d d^T (symmetric: the SYRK form, stored transposed)
    OzGemm gj{};
    gj.M = P; gj.N = P; gj.K = Q; gj.batch = 1; gj.S = S;
    gj.C = J_MO; gj.c_sb = 0; gj.c_r = lin(1); gj.c_c = lin(P);
    gj.sym = SYM_ROWCOL; gj.tag = "ozaki_tc:J_MO"; gj.tile_counter = w.ctr;
    GB_TRY(ozaki_gemm(w.dS, w.dS, gj, s));
    GB_TRY(launch_row_sumsq(w.bMO, K_MO, (long long)P * P, Q, s));
  }
  // w[b][l] = sum_q cj12[b][q] d[q][l] (diagonal of cj12 zero): rows l x orbitals b
  GB_TRY(launch_copy_zero_diag(cj12, w.cjm, P, s));
  GB_TRY(slice_operand(SliceSrc{w.cjm, 0, lin(P), lin(1), true}, w.cjS, s));
  OzGemm gw{};
  gw.M = Q; gw.N = P; gw.K = P; gw.batch = 1; gw.S = S;
  gw.C = w.w; gw.c_sb = 0; gw.c_r = lin(1); gw.c_c = lin(Q);
  gw.sym = SYM_NONE; gw.tag = "ozaki_tc:w"; gw.tile_counter = w.ctr;
  GB_TRY(ozaki_gemm(w.dT, w.cjS, gw, s));
  GB_TRY(launch_add_scaled_rows(w.w, w.d, n, P, Q, nbeta, nalpha, s));
  // the w term rides in the diagonal blocks of the exchange operand
  GB_TRY(launch_make_exchange_operand(w.bMO, ck12, w.w, w.Y, P, Q, s));
  // Z[m][b] = sum_(q,l) T[q][m][l] Y[b][q][l]; K = (q, l) cut into w.ns ranges
  // of whole orbitals (split s = batch s: its T block starts at orbital
  // s P / ns, element (m, k) at k / Q * N Q + m Q + k % Q; Y row b at b P Q + s kc + k)
  const long long qps = P / w.ns;  // orbitals per split
  GB_TRY(slice_operand(SliceSrc{w.Tf, qps * N * Q, lin(Q), split(Q, (long long)N * Q, 1), true}, w.Sx, s));
  GB_TRY(slice_operand(SliceSrc{w.Y, w.kc, lin((long long)P * Q), lin(1), true}, w.Sy, s));
  // rows m x orbitals b on the N tile (a ragged orbital count pads less there)
  OzGemm ge{};
  ge.M = N; ge.N = P; ge.K = w.kc; ge.batch = w.ns; ge.S = S;
  ge.sym = SYM_NONE; ge.tag = "ozaki_tc:ck_exchange"; ge.tile_counter = w.ctr;
  if (w.ns > 1) {
    ge.C = w.part; ge.c_sb = (long long)N * P; ge.c_r = lin(P); ge.c_c = lin(1);
    GB_TRY(ozaki_gemm(w.Sx, w.Sy, ge, s));
    const long long np = (long long)N * P;
    GB_LAUNCH("sum_splits", s,
              sum_splits_kernel<<<(unsigned)((np + 255) / 256), 256, 0, s>>>(w.part, w.ns, N, P, w.Z, P));
  } else {
    ge.C = w.Z; ge.c_sb = 0; ge.c_r = lin(P); ge.c_c = lin(1);
    GB_TRY(ozaki_gemm(w.Sx, w.Sy, ge, s));
  }
  // elag[a][b] = -sum_m C[m][a] Z[m][b] (b < nbf5), then the n_b Hmat term
  GB_TRY(slice_operand(SliceSrc{C, 0, lin(1), lin(N), false}, w.Ct, s));
  GB_TRY(slice_operand(SliceSrc{w.Z, 0, lin(1), lin(P), false}, w.Zt, s));
  OzGemm gz{};
  gz.M = N; gz.N = P; gz.K = N; gz.batch = 1; gz.S = S; gz.negate = 1;
  gz.C = elag; gz.c_sb = 0; gz.c_r = lin(N); gz.c_c = lin(1);
  gz.sym = SYM_NONE; gz.tag = "ozaki_tc:elag"; gz.tile_counter = w.ctr;
  GB_TRY(ozaki_gemm(w.Ct, w.Zt, gz, s));
  return launch_lagrange2_hterm(Hmat, n, elag, N, P, s);
}

int check_lagrange2_mixed(int N, int P, int Q, int nbeta, int nalpha, int S, const char* who) {
  GB_TRY(check_mixed(N, P, Q, S));
  GB_REQUIRE((long long)P * Q < 2147483647LL, GB_ERR_BAD_SHAPE, "%s: nbf5*naux too large", who);
  GB_REQUIRE(0 <= nbeta && nbeta <= nalpha && nalpha <= P, GB_ERR_BAD_SHAPE, "%s: need 0 <= nbeta <= nalpha <= nbf5",
             who);
  return GB_OK;
}
}  // namespace

extern "C" int gb_lagrange2_ri_mixed(const double* C, const double* H, const void* prep, const double* n,
                                     const double* cj12, const double* ck12, int nbf, int nbf5, int naux, int nbeta,
                                     int nalpha, int nslices, double* elag, double* Hmat, void* workspace,
                                     size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5, Q = naux, S = nslices;
  GB_TRY(check_lagrange2_mixed(N, P, Q, nbeta, nalpha, S, "gb_lagrange2_ri_mixed"));
  GB_REQUIRE(C && H && prep && n && cj12 && ck12 && elag && Hmat, GB_ERR_INVALID_ARG,
             "gb_lagrange2_ri_mixed: null pointer");
  GB_REQUIRE(workspace_bytes >= gb_lagrange2_ri_workspace_mixed(N, P, Q, S), GB_ERR_WORKSPACE,
             "gb_lagrange2_ri_mixed: workspace too small");
  return lagrange2_mixed_body(C, H, prep, n, cj12, ck12, N, P, Q, nbeta, nalpha, S, elag, Hmat, nullptr, nullptr,
                              nullptr, workspace, workspace_bytes, static_cast<cudaStream_t>(stream));
}

extern "C" size_t gb_jkh_lagrange2_ri_workspace_mixed(int nbf, int nbf5, int naux, int nslices) {
  return gb_lagrange2_ri_workspace_mixed(nbf, nbf5, naux, nslices);
}

extern "C" int gb_jkh_lagrange2_ri_mixed(const double* C, const double* H, const void* prep, const double* n,
                                         const double* cj12, const double* ck12, int nbf, int nbf5, int naux,
                                         int nbeta, int nalpha, int nslices, double* J_MO, double* K_MO,
                                         double* H_core, double* elag, double* Hmat, void* workspace,
                                         size_t workspace_bytes, void* stream) {
  clear_error();
  const int N = nbf, P = nbf5, Q = naux, S = nslices;
  GB_TRY(check_lagrange2_mixed(N, P, Q, nbeta, nalpha, S, "gb_jkh_lagrange2_ri_mixed"));
  GB_REQUIRE(C && H && prep && n && cj12 && ck12 && J_MO && K_MO && H_core && elag && Hmat, GB_ERR_INVALID_ARG,
             "gb_jkh_lagrange2_ri_mixed: null pointer");
  GB_REQUIRE(workspace_bytes >= gb_jkh_lagrange2_ri_workspace_mixed(N, P, Q, S), GB_ERR_WORKSPACE,
             "gb_jkh_lagrange2_ri_mixed: workspace too small");
  return lagrange2_mixed_body(C, H, prep, n, cj12, ck12, N, P, Q, nbeta, nalpha, S, elag, Hmat, J_MO, K_MO, H_core,
                              workspace, workspace_bytes, static_cast<cudaStream_t>(stream));
}
