// Digit slicing of FP64 operands for the split-product tensor-core path.
//
// A row x[0..K) of an FP64 operand is written as
//     x[k] = 2^E * sum_{s=1..S} d_s[k] 2^(-7 s)   (+ rounding error < 2^(E - 7S - 1))
// with E the row's power-of-two exponent (|x[k]| < 2^E for the whole row) and
// d_s balanced base-128 digits: |d_1| <= 128, |d_s| <= 64 for s >= 2.  Every
// digit is stored pre-weighted as the bf16 value d_s 2^(-7 s), which is exact
// (at most 8 significant bits).  Products of two slices then carry their
// positional weight, and a sum of slice products over a K-chunk is an integer
// multiple of 2^(-7 g) (g = s + t) that FP32 holds exactly while it stays below
// 2^24 units -- the property the tensor-core kernel relies on.
//
// The digits are computed from the FP64 bit pattern with integer arithmetic
// only (GB300's FP64 ALU rate is ~1/64 of FP32).
//
// Memory layout ("blocked"): the slices are stored in exactly the order the
// tensor-core kernel's shared memory wants them, so that one pipeline stage of
// one operand is a single contiguous bulk copy.  Rows are cut into blocks of
// 128 and K into blocks of 16; block (rb, kb) holds the S slice tiles of
// 128 x 16 bf16 back to back (4 KB each).  Inside a tile the 8 x 8 "core
// matrices" (8 rows of 16 bytes) are ordered k group major, row group minor,
// so the 16 core matrices of one k group are 2 KB of consecutive bytes:
//   byte(r, k) = ((k / 8) * 16 + r / 8) * 128 + (r % 8) * 16 + (k % 8) * 2.
// Blocks are ordered [batch][rb][kb].  Rows and K are zero-padded to whole
// blocks.  Exponents: exps[b][r] (int32).
//
// TF32x3 form (split code SPLIT_TF32X3): two planes, hi = tf32(x 2^-E) and
// lo = tf32(x 2^-E - hi) (each rounded to nearest even, 11 significant bits,
// FP32 exponent), for the classic three-product TF32 split (hi hi + hi lo +
// lo hi with FP32 accumulation).  A block is then 128 rows x 8 k of 32-bit
// elements, the same 4 KB tiles and core-matrix order with 4 elements per
// 16-byte core-matrix row:
//   byte(r, k) = ((k / 4) * 16 + r / 8) * 128 + (r % 8) * 16 + (k % 4) * 4.
#pragma once

#include <cuda_bf16.h>

#include "gemm_f64.cuh"

namespace gb {

constexpr int SL_ROWS = 128;               // rows per block
constexpr int SL_K = 16;                   // K per block
constexpr int SL_TILE_BYTES = SL_ROWS * SL_K * 2;  // one slice of one block: 4 KB

// Split codes ("nslices" in the C ABI): 1..6 bf16 digit slices, or the TF32x3 split.
constexpr int SPLIT_TF32X3 = 32;
struct SliceForm {
  int S, kind;  // planes; 0 = bf16 digits, 1 = tf32 hi/lo
};
__host__ __device__ inline bool valid_split(int code) { return (code >= 1 && code <= 6) || code == SPLIT_TF32X3; }
__host__ __device__ inline SliceForm form_of(int code) {
  return code == SPLIT_TF32X3 ? SliceForm{2, 1} : SliceForm{code, 0};
}

struct SliceSrc {
  const double* p;
  long long sb;  // batch stride
  Index2 r, k;   // row and K index maps
  bool kfast;    // K is the unit-stride index (else rows are)
  // > 0: the rows are the packed upper triangle of tri_n x tri_n index
  // pairs (tri_pair); row r reads r.at(m * tri_n + n)
  int tri_n = 0;
  __host__ __device__ __forceinline__ long long row_at(long long row) const {
    if (tri_n <= 0) return r.at(row);
    int m, n;
    tri_pair(row, tri_n, m, n);
    return r.at((long long)m * tri_n + n);
  }
};

struct SlicedDesc {
  __nv_bfloat16* planes;  // blocked digit tiles (32-bit elements when kind == 1)
  int* exps;              // [batch][rows]
  int batch, rows, K, S;
  int kind = 0;  // 0: bf16 digits, 16 k per block; 1: tf32 hi/lo, 8 k per block
  __host__ __device__ int kper() const { return kind ? SL_K / 2 : SL_K; }
  __host__ __device__ int code() const { return kind ? SPLIT_TF32X3 : S; }  // the split code it was cut with
  __host__ __device__ int rblocks() const { return (rows + SL_ROWS - 1) / SL_ROWS; }
  __host__ __device__ int kblocks() const { return (K + kper() - 1) / kper(); }
  __host__ __device__ long long block_bytes() const { return (long long)S * SL_TILE_BYTES; }
  __host__ __device__ long long batch_bytes() const { return (long long)rblocks() * kblocks() * block_bytes(); }
};

// `code` is a split code (1..6 or SPLIT_TF32X3).
inline size_t sliced_plane_bytes(int batch, int rows, int K, int code) {
  const SliceForm f = form_of(code);
  SlicedDesc d{nullptr, nullptr, batch, rows, K, f.S, f.kind};
  return (size_t)batch * d.batch_bytes();
}
inline size_t sliced_exp_bytes(int batch, int rows) { return (size_t)batch * rows * sizeof(int); }

// Carve a sliced operand (planes + exponents) out of a workspace or buffer.
template <class Cv>
SlicedDesc take_sliced(Cv& c, int batch, int rows, int K, int code) {
  auto* p = c.template take<unsigned char>(sliced_plane_bytes(batch, rows, K, code));
  auto* e = c.template take<int>((size_t)batch * rows);
  const SliceForm f = form_of(code);
  return SlicedDesc{reinterpret_cast<__nv_bfloat16*>(p), e, batch, rows, K, f.S, f.kind};
}

// Exponents then digits; both kernels read the source once.  With
// exps_ready the row exponents are already in dst.exps (recorded by the
// kernel that wrote the source) and only the digits are formed.
int slice_operand(const SliceSrc& src, const SlicedDesc& dst, cudaStream_t s, bool exps_ready = false);

}  // namespace gb
