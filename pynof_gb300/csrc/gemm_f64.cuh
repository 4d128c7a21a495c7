// FP64 contraction engine (DMMA m8n8k4) used by the plain FP64 path.
//
// One batched GEMM  C[b](i, j) = alpha * sum_k A[b](i, k) B[b](k, j) + beta * C[b](i, j)
// whose operands are addressed through "split" index maps: an index r maps to
//   (r / div) * s1 + (r % div) * s0          (div == 0 means  r * s0)
// which covers plain strided matrices and the 4-index views the full-ERI
// exchange build needs (rows (m, s), columns (n, l) of (mn|sl)).
//
// Symmetry modes skip redundant tiles and mirror the results:
//   SYM_NONE     every tile computed and stored;
//   SYM_ROWCOL   square output symmetric in (i, j): tiles below the diagonal
//                are skipped, off-diagonal tiles are also written transposed;
//   SYM_PAIRCOL  columns encode an index pair j = m * pair_n + n and the
//                output is symmetric in (m, n): tiles whose every column has
//                n < m are skipped, columns with n > m are also written to
//                n * pair_n + m.
#pragma once

#include "gb_common.cuh"

namespace gb {

struct Index2 {
  long long div, s1, s0;
  __host__ __device__ __forceinline__ long long at(long long r) const {
    return div ? (r / div) * s1 + (r % div) * s0 : r * s0;
  }
};

struct MatF64 {
  const double* p;
  long long sb;  // batch stride (elements)
  Index2 r, c;   // row / column index maps
};

struct OutF64 {
  double* p;
  long long sb;
  Index2 r, c;
};

// SYM_TRIROW / SYM_TRICOL (tensor-core path only, where they replace
// SYM_PAIRCOL): rows (columns) are the packed upper triangle of the pairs,
// r -> (m, n) with m <= n (tri_pair), pair_n (pair_n + 1) / 2 of them; the
// output at pair m * pair_n + n is written, and for n > m also its mirror
// n * pair_n + m.
enum SymMode { SYM_NONE = 0, SYM_ROWCOL = 1, SYM_PAIRCOL = 2, SYM_TRIROW = 4, SYM_TRICOL = 5 };

// Packed upper-triangle index r = m N - m (m - 1) / 2 + (n - m), 0 <= m <= n < N,
// back to (m, n) (rows of the triangle in order, each from its diagonal on).
__host__ __device__ __forceinline__ void tri_pair(long long r, int N, int& m, int& n) {
  const double b = 2.0 * N + 1.0;
  long long x = (long long)((b - sqrt(b * b - 8.0 * (double)r)) * 0.5);
  x = x < 0 ? 0 : (x > N - 1 ? N - 1 : x);
  while (x > 0 && x * N - x * (x - 1) / 2 > r) --x;
  while (x + 1 < N && (x + 1) * N - (x + 1) * x / 2 <= r) ++x;
  m = (int)x;
  n = (int)(r - (x * N - x * (x - 1) / 2) + x);
}

struct GemmF64 {
  int M, N, K, batch;
  MatF64 A;  // M x K
  MatF64 B;  // K x N
  OutF64 C;  // M x N
  double alpha, beta;
  int sym;
  int pair_n;
  bool a_kfast;  // A's K index is the unit-stride one (coalesced along k)
  bool b_kfast;  // B's K index is the unit-stride one
  const char* tag = "gemm_f64";  // profiler label
};

// Plain strided helpers ---------------------------------------------------
inline Index2 lin(long long s) { return Index2{0, 0, s}; }
inline Index2 split(long long div, long long s1, long long s0) { return Index2{div, s1, s0}; }

int gemm_f64(const GemmF64& g, cudaStream_t stream);

}  // namespace gb
