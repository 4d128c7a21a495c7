// Digit slicing of FP64 operands (see slice.cuh for the representation).
#include "slice.cuh"

namespace gb {
namespace {

constexpr int TILE = 32;

__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}

// |x| < 2^E for every x whose |bits| <= maxbits (order of |x| == order of its bits).
__device__ __forceinline__ int exponent_of(unsigned long long maxbits) {
  const int ex = (int)(maxbits >> 52);
  return (ex == 0 ? 1 : ex) - 1022;
}

// Balanced base-128 digits of round(x 2^(7S - E)), stored pre-weighted.
__device__ __forceinline__ void make_digits(double x, int E, int S, __nv_bfloat16* out) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  int ex = (int)((bits >> 52) & 0x7FF);
  unsigned long long m = bits & 0xFFFFFFFFFFFFFull;
  if (ex) m |= 1ull << 52; else ex = 1;
  const int r = 1075 + E - ex - 7 * S;  // right shift of the 53-bit mantissa (>= 11 for S <= 6)
  long long xi;
  if (r <= 0) xi = (long long)(m << (-r));
  else if (r >= 64) xi = 0;
  else xi = (long long)((m + (1ull << (r - 1))) >> r);
  if (bits >> 63) xi = -xi;
  float w = 1.0f;
#pragma unroll 1
  for (int s = 0; s < S; ++s) w *= 0.0078125f;  // 2^(-7S)
#pragma unroll 1
  for (int s = S; s >= 2; --s) {
    const long long d = ((xi + 64) & 127) - 64;
    xi = (xi - d) >> 7;
    out[s - 1] = __float2bfloat16_rn((float)d * w);
    w *= 128.0f;
  }
  out[0] = __float2bfloat16_rn((float)xi * w);
}

// One warp per row; K is the unit-stride index.
__global__ void rowexp_kfast_kernel(SliceSrc src, int rows, int K, int* __restrict__ exps) {
  const long long b = blockIdx.y;
  const long long row = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= rows) return;
  const double* base = src.p + b * src.sb + src.r.at(row);
  unsigned long long mx = 0;
  for (int k = lane; k < K; k += 32) {
    const unsigned long long v = abs_bits(base[src.k.at(k)]);
    mx = v > mx ? v : mx;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = v > mx ? v : mx;
  }
  if (lane == 0) exps[b * rows + row] = exponent_of(mx);
}

// One thread per row; rows are the unit-stride index.
__global__ void rowexp_rfast_kernel(SliceSrc src, int rows, int K, int* __restrict__ exps) {
  const long long b = blockIdx.y;
  const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= rows) return;
  const double* base = src.p + b * src.sb + src.r.at(row);
  unsigned long long mx = 0;
  for (int k = 0; k < K; ++k) {
    const unsigned long long v = abs_bits(base[src.k.at(k)]);
    mx = v > mx ? v : mx;
  }
  exps[b * rows + row] = exponent_of(mx);
}

// 32 x 32 tiles, 32 x 8 threads.  KFAST: load and store along k directly.
// Otherwise load along rows, transpose through shared memory, store along k.
template <bool KFAST>
__global__ void digits_kernel(SliceSrc src, SlicedDesc dst, int tiles_k) {
  __shared__ __nv_bfloat16 sm[KFAST ? 1 : 6][TILE][TILE + 2];
  const long long b = blockIdx.y;
  const int tr = blockIdx.x / tiles_k, tk = blockIdx.x % tiles_k;
  const int r0 = tr * TILE, k0 = tk * TILE;
  const int S = dst.S;
  const double* base = src.p + b * src.sb;
  const int* ex = dst.exps + b * dst.rows;
  __nv_bfloat16* planes = dst.planes + b * (long long)S * dst.rows * dst.kpad;
  const long long plane_stride = (long long)dst.rows * dst.kpad;
  __nv_bfloat16 dg[6];
  if (KFAST) {
    const int k = k0 + threadIdx.x;
    for (int i = threadIdx.y; i < TILE; i += blockDim.y) {
      const int r = r0 + i;
      if (r >= dst.rows || k >= dst.kpad) continue;
      double x = 0.0;
      if (k < dst.K) x = base[src.r.at(r) + src.k.at(k)];
      make_digits(x, ex[r], S, dg);
      __nv_bfloat16* o = planes + (long long)r * dst.kpad + k;
      for (int s = 0; s < S; ++s) o[s * plane_stride] = dg[s];
    }
  } else {
    const int r = r0 + threadIdx.x;
    for (int i = threadIdx.y; i < TILE; i += blockDim.y) {
      const int k = k0 + i;
      double x = 0.0;
      int e = 0;
      if (r < dst.rows) {
        e = ex[r];
        if (k < dst.K) x = base[src.r.at(r) + src.k.at(k)];
      }
      make_digits(x, e, S, dg);
      for (int s = 0; s < S; ++s) sm[s][i][threadIdx.x] = dg[s];
    }
    __syncthreads();
    const int k = k0 + threadIdx.x;
    for (int i = threadIdx.y; i < TILE; i += blockDim.y) {
      const int rr = r0 + i;
      if (rr >= dst.rows || k >= dst.kpad) continue;
      __nv_bfloat16* o = planes + (long long)rr * dst.kpad + k;
      for (int s = 0; s < S; ++s) o[s * plane_stride] = sm[s][threadIdx.x][i];
    }
  }
}

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

int slice_operand(const SliceSrc& src, const SlicedDesc& dst, cudaStream_t s) {
  GB_REQUIRE(dst.S >= 1 && dst.S <= 6, GB_ERR_INVALID_ARG, "slice_operand: nslices=%d outside [1, 6]", dst.S);
  GB_REQUIRE(dst.kpad == slice_kpad(dst.K), GB_ERR_INVALID_ARG, "slice_operand: kpad mismatch");
  GB_REQUIRE(dst.batch >= 1 && dst.batch <= 65535 && dst.rows >= 0, GB_ERR_BAD_SHAPE, "slice_operand: bad batch");
  if (dst.rows == 0 || dst.K == 0) return GB_OK;
  if (src.kfast) {
    GB_LAUNCH("slice_rowexp", s,
              rowexp_kfast_kernel<<<dim3(cdiv(dst.rows, 8), dst.batch), 256, 0, s>>>(src, dst.rows, dst.K, dst.exps));
  } else {
    GB_LAUNCH("slice_rowexp", s,
              rowexp_rfast_kernel<<<dim3(cdiv(dst.rows, 256), dst.batch), 256, 0, s>>>(src, dst.rows, dst.K, dst.exps));
  }
  const long long tiles_k = cdiv(dst.kpad, TILE);
  const long long tiles = cdiv(dst.rows, TILE) * tiles_k;
  GB_REQUIRE(tiles <= 2147483647LL, GB_ERR_BAD_SHAPE, "slice_operand: too many tiles");
  if (src.kfast) {
    GB_LAUNCH("slice_digits", s,
              digits_kernel<true><<<dim3((unsigned)tiles, dst.batch), dim3(TILE, 8), 0, s>>>(src, dst, (int)tiles_k));
  } else {
    GB_LAUNCH("slice_digits", s,
              digits_kernel<false><<<dim3((unsigned)tiles, dst.batch), dim3(TILE, 8), 0, s>>>(src, dst, (int)tiles_k));
  }
  return GB_OK;
}

}  // namespace gb
