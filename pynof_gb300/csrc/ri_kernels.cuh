// Bandwidth-bound helper kernels of the FP64 RI path (reductions, gathers,
// elementwise weights).  All launchers return a GB_* status.
#pragma once

#include "gb_common.cuh"

namespace gb {

// d[q][l] = sum_n C[n][q] T[q][n][l]
// d[q][l] = sum_n C[n][q] T[q][n][l]; with texps also the row exponents of
// T's digit slicing with rows (q, n) and K = l (texps[q N + n]).
int launch_contract_diag(const double* C, const double* T, double* d, int N, int P, int Q, cudaStream_t s,
                         int* texps = nullptr);
// d[p][l] = src[p * stride_pp + l]
int launch_gather_diag(const double* src, double* d, int P, int Q, long long stride_pp, cudaStream_t s);
// out[r] = sum_l src[r][l]^2
int launch_row_sumsq(const double* src, double* out, long long rows, int Q, cudaStream_t s);
// out[p] = sum_m C[m * ldc + p] X[m * ldx + p]
int launch_col_dot(const double* C, int ldc, const double* X, int ldx, double* out, int N, int P,
                   cudaStream_t s);
// dst = src with the diagonal set to zero (P x P)
int launch_copy_zero_diag(const double* src, double* dst, int P, cudaStream_t s);
// w[b][k] += coef_b d[b][k], coef_b = n[b] for b < nbeta or b >= nalpha, else 0
int launch_add_scaled_rows(double* w, const double* d, const double* n, int P, int Q, int nbeta, int nalpha,
                           cudaStream_t s);
// Y[b][q][k] = (q != b) ck12[b][q] bMO[b][q][k]
int launch_make_ck_weighted(const double* bMO, const double* ck12, double* Y, int P, int Q, cudaStream_t s);
// Y[b][q][k] = ck12[b][q] bMO[b][q][k] (q != b), -w[b][k] (q == b): the exchange
// operand of the tensor-core Lagrangian with the w term folded into its diagonal block
int launch_make_exchange_operand(const double* bMO, const double* ck12, const double* w, double* Y, int P, int Q,
                                 cudaStream_t s);
// elag[a][b] += n[b] Hmat[a][b] (b < P); elag[a][b] = 0 (b >= P)
int launch_lagrange2_hterm(const double* Hmat, const double* n, double* elag, int N, int P, cudaStream_t s);
// elag[a][b] += n[b] Hmat[a][b] + sum_k bMO[a][b][k] w[b][k] (b < P); elag[a][b] = 0 (b >= P)
int launch_lagrange2_finish(const double* bMO, const double* w, const double* Hmat, const double* n,
                            double* elag, int N, int P, int Q, cudaStream_t s);

}  // namespace gb
