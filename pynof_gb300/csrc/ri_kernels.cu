// Bandwidth-bound helper kernels of the FP64 RI path.
#include "ri_kernels.cuh"

namespace gb {
namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void contract_diag_kernel(const double* __restrict__ C, const double* __restrict__ T,
                                     double* __restrict__ d, int N, int P, int Q) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  const int q = blockIdx.y;
  if (l >= Q) return;
  const double* Tq = T + (long long)q * N * Q + l;
  double acc = 0.0;
  for (int n = 0; n < N; ++n) acc = fma(__ldg(C + (long long)n * N + q), __ldg(Tq + (long long)n * Q), acc);
  d[(long long)q * Q + l] = acc;
}

// The same contraction, also recording the row exponents of T's digit
// slicing with rows (q, n) and K = l: texps[q N + n] = E with
// |T[q][n][l]| < 2^E for all l (entries preset below any E).  A warp holds 32
// consecutive l; the exponent field's maximum over them comes from one warp
// reduction per n and lands in lane n % 32, which folds it in with atomicMax
// every 32 n.
// A NaN or an infinity in T (exponent field 0x7FF) is reported in the status
// word, as the slicer does for the rows it measures.
__global__ void contract_diag_exps_kernel(const double* __restrict__ C, const double* __restrict__ T,
                                          double* __restrict__ d, int* __restrict__ texps, int N, int P, int Q,
                                          int* status) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  const int q = blockIdx.y;
  const int lane = threadIdx.x & 31;
  const bool in = l < Q;  // the whole warp stays for the reductions
  const double* Tq = T + (long long)q * N * Q + (in ? l : 0);
  int* eq = texps + (long long)q * N;
  double acc = 0.0;
  unsigned int mine = 0;  // exponent field maximum of row n0 + lane
  for (int n0 = 0; n0 < N; n0 += 32) {
    const int nn = min(32, N - n0);
    for (int j = 0; j < nn; ++j) {
      const int n = n0 + j;
      const double t = in ? __ldg(Tq + (long long)n * Q) : 0.0;
      acc = fma(__ldg(C + (long long)n * N + q), t, acc);
      const unsigned int ex = (unsigned int)((unsigned long long)__double_as_longlong(t) >> 52) & 0x7FFu;
      const unsigned int mx = __reduce_max_sync(0xffffffffu, ex);
      if (lane == j) mine = mx;
    }
    if (lane < nn) {
      atomicMax(eq + n0 + lane, (int)(mine > 1u ? mine : 1u) - 1022);
      if (mine == 0x7FFu && status) atomicCAS(status, 0, GB_ERR_NONFINITE);
    }
  }
  if (in) d[(long long)q * Q + l] = acc;
}

__global__ void gather_diag_kernel(const double* __restrict__ src, double* __restrict__ d, int Q,
                                   long long stride_pp) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y;
  if (l < Q) d[(long long)p * Q + l] = src[(long long)p * stride_pp + l];
}

// one warp per row
__global__ void row_sumsq_kernel(const double* __restrict__ src, double* __restrict__ out, long long rows,
                                 int Q) {
  const long long r = (long long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= rows) return;
  const double* s = src + r * Q;
  double acc = 0.0;
  for (int l = lane; l < Q; l += 32) {
    const double v = s[l];
    acc = fma(v, v, acc);
  }
  acc = warp_sum(acc);
  if (lane == 0) out[r] = acc;
}

__global__ void col_dot_kernel(const double* __restrict__ C, int ldc, const double* __restrict__ X, int ldx,
                               double* __restrict__ out, int N, int P) {
  const int p = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (p >= P) return;
  double acc = 0.0;
  for (int m = lane; m < N; m += 32) acc = fma(C[(long long)m * ldc + p], X[(long long)m * ldx + p], acc);
  acc = warp_sum(acc);
  if (lane == 0) out[p] = acc;
}

__global__ void copy_zero_diag_kernel(const double* __restrict__ src, double* __restrict__ dst, int P) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)P * P) return;
  const int r = (int)(i / P), c = (int)(i % P);
  dst[i] = (r == c) ? 0.0 : src[i];
}

__global__ void add_scaled_rows_kernel(double* __restrict__ w, const double* __restrict__ d,
                                       const double* __restrict__ n, int P, int Q, int nbeta, int nalpha) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (k >= Q) return;
  if (b < nbeta || b >= nalpha) {
    const long long i = (long long)b * Q + k;
    w[i] = fma(n[b], d[i], w[i]);
  }
}

__global__ void make_ck_weighted_kernel(const double* __restrict__ bMO, const double* __restrict__ ck12,
                                        double* __restrict__ Y, int P, int Q) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int q = blockIdx.y;
  const int b = blockIdx.z;
  if (k >= Q) return;
  const long long i = ((long long)b * P + q) * Q + k;
  const double c = (q == b) ? 0.0 : ck12[(long long)b * P + q];
  Y[i] = c * bMO[i];
}

// one warp per (a, b) with b < P; blocks past the dot range zero elag[:, P:]
__global__ void lagrange2_finish_kernel(const double* __restrict__ bMO, const double* __restrict__ w,
                                        const double* __restrict__ Hmat, const double* __restrict__ n,
                                        double* __restrict__ elag, int N, int P, int Q) {
  const long long pair = (long long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (pair >= (long long)N * P) return;
  const int a = (int)(pair / P), b = (int)(pair % P);
  const double* x = bMO + ((long long)a * P + b) * Q;
  const double* y = w + (long long)b * Q;
  double acc = 0.0;
  for (int k = lane; k < Q; k += 32) acc = fma(x[k], y[k], acc);
  acc = warp_sum(acc);
  if (lane == 0) {
    double* e = elag + (long long)a * N + b;
    *e = *e + n[b] * Hmat[(long long)a * P + b] + acc;
  }
}

// Exchange operand of the tensor-core Lagrangian: Y[b][q][k] = ck12[b][q]
// bMO[b][q][k] for q != b and -w[b][k] on the diagonal block q == b, so that
// -sum_(q,k) bMO[a][q][k] Y[b][q][k] also carries + sum_k bMO[a][b][k] w[b][k].
// Grid-stride over (b, q) rows of Q; two elements per thread and step
// (16-byte accesses when Q is even).
__global__ void make_exchange_operand_kernel(const double* __restrict__ bMO, const double* __restrict__ ck12,
                                             const double* __restrict__ w, double* __restrict__ Y, int P, int Q) {
  const long long rows = (long long)P * P;
  const int half = Q >> 1;
  const bool even = (Q & 1) == 0;
  for (long long row = blockIdx.x; row < rows; row += gridDim.x) {
    const int b = (int)(row / P), q = (int)(row % P);
    const bool diag = q == b;
    const double c = diag ? -1.0 : ck12[(long long)b * P + q];
    const double* src = diag ? w + (long long)b * Q : bMO + row * Q;
    double* dst = Y + row * Q;
    if (even) {
      for (int k2 = threadIdx.x; k2 < half; k2 += blockDim.x) {
        const double2 v = __ldcs(reinterpret_cast<const double2*>(src) + k2);
        __stcs(reinterpret_cast<double2*>(dst) + k2, make_double2(c * v.x, c * v.y));
      }
    } else {
      for (int k = threadIdx.x; k < Q; k += blockDim.x) dst[k] = c * src[k];
    }
  }
}

// elag[a][b] += n[b] Hmat[a][b] for b < P; elag[a][b] = 0 for b >= P
__global__ void lagrange2_hterm_kernel(const double* __restrict__ Hmat, const double* __restrict__ n,
                                       double* __restrict__ elag, int N, int P) {
  const long long total = (long long)N * N;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(i / N), b = (int)(i % N);
    elag[i] = b < P ? elag[i] + n[b] * Hmat[(long long)a * P + b] : 0.0;
  }
}

__global__ void zero_tail_cols_kernel(double* __restrict__ elag, int N, int P) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int W = N - P;
  if (i >= (long long)N * W) return;
  const int a = (int)(i / W), c = P + (int)(i % W);
  elag[(long long)a * N + c] = 0.0;
}

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

int launch_contract_diag(const double* C, const double* T, double* d, int N, int P, int Q, cudaStream_t s,
                         int* texps) {
  if (texps) {
    // every entry below any exponent folded in (0x80808080 < -1021)
    GB_TRY(cuda_status(cudaMemsetAsync(texps, 0x80, sizeof(int) * (size_t)P * N, s), "contract_diag exponents"));
    GB_LAUNCH("contract_diag", s,
              contract_diag_exps_kernel<<<dim3(cdiv(Q, 128), P), 128, 0, s>>>(C, T, d, texps, N, P, Q,
                                                                               device_status_word()));
    return GB_OK;
  }
  GB_LAUNCH("contract_diag", s, contract_diag_kernel<<<dim3(cdiv(Q, 128), P), 128, 0, s>>>(C, T, d, N, P, Q));
  return GB_OK;
}

int launch_gather_diag(const double* src, double* d, int P, int Q, long long stride_pp, cudaStream_t s) {
  GB_LAUNCH("gather_diag", s, gather_diag_kernel<<<dim3(cdiv(Q, 128), P), 128, 0, s>>>(src, d, Q, stride_pp));
  return GB_OK;
}

int launch_row_sumsq(const double* src, double* out, long long rows, int Q, cudaStream_t s) {
  if (rows <= 0) return GB_OK;
  GB_LAUNCH("row_sumsq", s, row_sumsq_kernel<<<cdiv(rows, 8), 256, 0, s>>>(src, out, rows, Q));
  return GB_OK;
}

int launch_col_dot(const double* C, int ldc, const double* X, int ldx, double* out, int N, int P,
                   cudaStream_t s) {
  GB_LAUNCH("col_dot", s, col_dot_kernel<<<cdiv(P, 8), 256, 0, s>>>(C, ldc, X, ldx, out, N, P));
  return GB_OK;
}

int launch_copy_zero_diag(const double* src, double* dst, int P, cudaStream_t s) {
  GB_LAUNCH("copy_zero_diag", s, copy_zero_diag_kernel<<<cdiv((long long)P * P, 256), 256, 0, s>>>(src, dst, P));
  return GB_OK;
}

int launch_add_scaled_rows(double* w, const double* d, const double* n, int P, int Q, int nbeta, int nalpha,
                           cudaStream_t s) {
  GB_LAUNCH("add_scaled_rows", s, add_scaled_rows_kernel<<<dim3(cdiv(Q, 128), P), 128, 0, s>>>(w, d, n, P, Q, nbeta, nalpha));
  return GB_OK;
}

int launch_make_ck_weighted(const double* bMO, const double* ck12, double* Y, int P, int Q, cudaStream_t s) {
  GB_LAUNCH("make_ck_weighted", s, make_ck_weighted_kernel<<<dim3(cdiv(Q, 128), P, P), 128, 0, s>>>(bMO, ck12, Y, P, Q));
  return GB_OK;
}

int launch_make_exchange_operand(const double* bMO, const double* ck12, const double* w, double* Y, int P, int Q,
                                 cudaStream_t s) {
  const long long rows = (long long)P * P;
  if (rows == 0 || Q == 0) return GB_OK;
  const unsigned grid = (unsigned)(rows < 152LL * 16 ? rows : 152LL * 16);
  GB_LAUNCH("make_exchange_operand", s,
            make_exchange_operand_kernel<<<grid, 256, 0, s>>>(bMO, ck12, w, Y, P, Q));
  return GB_OK;
}

int launch_lagrange2_hterm(const double* Hmat, const double* n, double* elag, int N, int P, cudaStream_t s) {
  const long long total = (long long)N * N;
  if (total == 0) return GB_OK;
  const unsigned grid = (unsigned)(cdiv(total, 256) < 152u * 8 ? cdiv(total, 256) : 152u * 8);
  GB_LAUNCH("lagrange2_hterm", s, lagrange2_hterm_kernel<<<grid, 256, 0, s>>>(Hmat, n, elag, N, P));
  return GB_OK;
}

int launch_lagrange2_finish(const double* bMO, const double* w, const double* Hmat, const double* n,
                            double* elag, int N, int P, int Q, cudaStream_t s) {
  GB_LAUNCH("lagrange2_finish", s, lagrange2_finish_kernel<<<cdiv((long long)N * P, 8), 256, 0, s>>>(bMO, w, Hmat, n, elag, N, P, Q));
  if (N > P) {
    GB_LAUNCH("zero_tail_cols", s, zero_tail_cols_kernel<<<cdiv((long long)N * (N - P), 256), 256, 0, s>>>(elag, N, P));
  }
  return GB_OK;
}

}  // namespace gb
