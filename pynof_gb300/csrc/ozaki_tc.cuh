// Split-product FP64 GEMM on the tcgen05 tensor cores (bf16 digit slices).
//
// C[b](i, j) = (-1)^negate * sum_k A[b](i, k) B[b](j, k)
// with A, B given as digit slices (slice.cuh).  The slice products are grouped
// by g = s + t (uniform weight 2^(-7 g) inside a group).  Groups g <= 4 are the
// leading ones: they accumulate in FP32 TMEM over chunks of 192 k, where every
// partial sum is an integer multiple of 2^(-7 g) below 2^22 units and hence
// exact, and are drained into per-element int64 accumulators after each
// chunk.  Groups 5..S+1 (2^(-21) and less relative to the leading group)
// accumulate together in one FP32 accumulator over the whole K.  The epilogue
// assembles the FP64 result from the int64 and FP32 parts with integer
// arithmetic only.  Products with s + t > S + 1 are not formed.
//
// Accuracy: each element carries the slicing error (|x| 2^(-7 S - 1) per
// operand element relative to its row's power-of-two bound) plus the
// truncation of the product triangle; with S = 6 the result agrees with FP64
// to ~1e-12 normwise on the path's operands.  S = 2 is the classic
// three-product bf16x3 split.
#pragma once

#include "gemm_f64.cuh"
#include "slice.cuh"

namespace gb {

struct OzGemm {
  int M, N, K, batch, S;
  double* C;
  long long c_sb;
  Index2 c_r, c_c;
  int sym, pair_n;
  int negate;
  // Drain the FP32 accumulator of the small slice groups into the int64 fixed
  // point after every 192-k chunk (instead of once at the end): its rounding
  // error then stops growing with K.  Costs the overlap of the drain with
  // the MMAs; used for long contractions (K > 4096).
  int fdrain = 0;
  int bn = 128;  // N tile width: 32, 64 or 128 (128 required for SYM_ROWCOL)
  // Device word (caller memory, zeroed here before each launch that uses it)
  // from which the persistent form hands out tiles in order; null = a static
  // round-robin walk.  Launches that share it must be ordered (one stream).
  unsigned int* tile_counter = nullptr;
  const char* tag = "ozaki_tc";
};

// One GEMM of a grouped launch.
struct OzProblem {
  SlicedDesc A, B;
  OzGemm g;
};

// A: rows are the M index; B: rows are the N index; both K-major slices.
int ozaki_gemm(const SlicedDesc& A, const SlicedDesc& B, const OzGemm& g, cudaStream_t stream);

// Several GEMMs (same slice count and N tile width) in one launch.  `table`
// is caller device memory of ozaki_group_table_bytes(n) bytes; it is filled
// here with a synchronous copy, so a grouped launch can be captured into a
// CUDA graph once the table holds the problem list.
// With `persistent` set by the upload (every output's tile rows are its unit
// stride, bf16 digits, 128-wide tiles) and passed to the launch, the group
// runs as one persistent launch (one CTA per SM) walking the concatenated
// tile space in order through a counter in the table; otherwise one CTA per tile.
size_t ozaki_group_table_bytes(int nprob);
int ozaki_group_upload(const OzProblem* probs, int nprob, void* table, bool* persistent = nullptr);
int ozaki_gemm_grouped(const void* table, int nprob, long long total_tiles, int S, int bn, cudaStream_t stream,
                       const char* tag, bool persistent = false);
// Tiles of one problem (for building the grouped tile ranges).
long long ozaki_tiles(const OzGemm& g);

// Device status word of the tensor-core kernels (0 = ok, GB_ERR_TIMEOUT when a
// bounded wait gave up).  Reading synchronises the current device.
int ozaki_status(int reset, int* out);

// Launch attributes of the kernel (registers, limits, occupancy) as text.
int ozaki_kernel_info(char* out, size_t len);

}  // namespace gb
