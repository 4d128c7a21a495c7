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
// Plane layout: planes[b][s][r][kp] (bf16, row pitch kp = K rounded up to 8),
// exponents exps[b][r] (int32).
#pragma once

#include <cuda_bf16.h>

#include "gemm_f64.cuh"

namespace gb {

struct SliceSrc {
  const double* p;
  long long sb;  // batch stride
  Index2 r, k;   // row and K index maps
  bool kfast;    // K is the unit-stride index (else rows are)
};

struct SlicedDesc {
  __nv_bfloat16* planes;  // [batch][S][rows][kpad]
  int* exps;              // [batch][rows]
  int batch, rows, K, kpad, S;
};

inline int slice_kpad(int K) { return (K + 7) & ~7; }
inline size_t sliced_plane_bytes(int batch, int rows, int K, int S) {
  return (size_t)batch * S * rows * slice_kpad(K) * sizeof(__nv_bfloat16);
}
inline size_t sliced_exp_bytes(int batch, int rows) { return (size_t)batch * rows * sizeof(int); }

// Exponents then digits; both kernels read the source once.
int slice_operand(const SliceSrc& src, const SlicedDesc& dst, cudaStream_t s);

}  // namespace gb
