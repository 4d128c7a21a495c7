// Digit slicing of FP64 operands (see slice.cuh for the representation).
#include "slice.cuh"

namespace gb {
namespace {

__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}

// |x| < 2^E for every x whose |bits| <= maxbits (order of |x| == order of its bits).
__device__ __forceinline__ int exponent_of(unsigned long long maxbits) {
  const int ex = (int)(maxbits >> 52);
  return (ex == 0 ? 1 : ex) - 1022;
}

// Balanced base-128 digits of round(x 2^(7S - E)), stored pre-weighted as bf16
// bit patterns.  Every digit value d 2^(-7 s) (|d| <= 128) is exact in bf16, so
// its bf16 bits are the upper half of its FP32 bits; FP32 values come from
// the integer with the 1.5 * 2^23 magic-number trick (exact for |d| < 2^22).
template <int S>
__device__ __forceinline__ void make_digits(double x, int E, unsigned short* out) {
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
#pragma unroll
  for (int s = S; s >= 2; --s) {
    const int d = (((int)xi + 64) & 127) - 64;
    xi = (xi - d) >> 7;
    const float f = (__int_as_float(0x4B400000 + d) - 12582912.0f) * __int_as_float((127 - 7 * s) << 23);
    out[s - 1] = (unsigned short)(__float_as_uint(f) >> 16);
  }
  const float f1 = (__int_as_float(0x4B400000 + (int)xi) - 12582912.0f) * __int_as_float((127 - 7) << 23);
  out[0] = (unsigned short)(__float_as_uint(f1) >> 16);
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

// One CTA of 256 threads per (row block, k block): thread -> (row r, k group of
// 8).  Lanes 0..7 take consecutive rows of one core matrix and a warp covers
// 32 consecutive rows of one k group, i.e. four whole consecutive core
// matrices (512 contiguous bytes) per slice, written with 16-byte stores; it
// reads 64 contiguous source bytes per row (K-fast sources) or 256 contiguous
// bytes per k (row-fast sources).
template <int S>
__global__ void __launch_bounds__(256) digits_blocked_kernel(SliceSrc src, SlicedDesc dst) {
  const long long b = blockIdx.y;
  const int kbn = dst.kblocks();
  const int rb = blockIdx.x / kbn, kb = blockIdx.x % kbn;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ri = lane & 7, kg = warp >> 2, rg = (warp & 3) * 4 + (lane >> 3);
  const int r = rb * SL_ROWS + rg * 8 + ri;
  const int k0 = kb * SL_K + kg * 8;
  unsigned short dg[8][S];
  const bool rok = r < dst.rows;
  const double* base = src.p + b * src.sb + (rok ? src.r.at(r) : 0);
  const int e = rok ? dst.exps[b * dst.rows + r] : 0;
  double xs[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int k = k0 + u;
    xs[u] = (rok && k < dst.K) ? base[src.k.at(k)] : 0.0;
  }
#pragma unroll
  for (int u = 0; u < 8; ++u) make_digits<S>(xs[u], e, dg[u]);
  unsigned char* out = reinterpret_cast<unsigned char*>(dst.planes) + b * dst.batch_bytes() +
                       ((long long)blockIdx.x * S) * SL_TILE_BYTES + (kg * 16 + rg) * 128 + ri * 16;
#pragma unroll
  for (int s = 0; s < S; ++s) {
    uint4 v;
    v.x = (unsigned)dg[0][s] | ((unsigned)dg[1][s] << 16);
    v.y = (unsigned)dg[2][s] | ((unsigned)dg[3][s] << 16);
    v.z = (unsigned)dg[4][s] | ((unsigned)dg[5][s] << 16);
    v.w = (unsigned)dg[6][s] | ((unsigned)dg[7][s] << 16);
    *reinterpret_cast<uint4*>(out + (long long)s * SL_TILE_BYTES) = v;
  }
}

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

int slice_operand(const SliceSrc& src, const SlicedDesc& dst, cudaStream_t s) {
  GB_REQUIRE(dst.S >= 1 && dst.S <= 6, GB_ERR_INVALID_ARG, "slice_operand: nslices=%d outside [1, 6]", dst.S);
  GB_REQUIRE(dst.batch >= 1 && dst.batch <= 65535 && dst.rows >= 0, GB_ERR_BAD_SHAPE, "slice_operand: bad batch");
  GB_REQUIRE((reinterpret_cast<uintptr_t>(dst.planes) & 15) == 0, GB_ERR_INVALID_ARG,
             "slice_operand: planes not 16-byte aligned");
  if (dst.rows == 0 || dst.K == 0) return GB_OK;
  if (src.kfast) {
    GB_LAUNCH("slice_rowexp", s,
              rowexp_kfast_kernel<<<dim3(cdiv(dst.rows, 8), dst.batch), 256, 0, s>>>(src, dst.rows, dst.K, dst.exps));
  } else {
    GB_LAUNCH("slice_rowexp", s,
              rowexp_rfast_kernel<<<dim3(cdiv(dst.rows, 256), dst.batch), 256, 0, s>>>(src, dst.rows, dst.K, dst.exps));
  }
  const long long blocks = (long long)dst.rblocks() * dst.kblocks();
  GB_REQUIRE(blocks <= 2147483647LL, GB_ERR_BAD_SHAPE, "slice_operand: too many blocks");
  const dim3 grid((unsigned)blocks, dst.batch);
  switch (dst.S) {
    case 1: GB_LAUNCH("slice_digits", s, digits_blocked_kernel<1><<<grid, 256, 0, s>>>(src, dst)); break;
    case 2: GB_LAUNCH("slice_digits", s, digits_blocked_kernel<2><<<grid, 256, 0, s>>>(src, dst)); break;
    case 3: GB_LAUNCH("slice_digits", s, digits_blocked_kernel<3><<<grid, 256, 0, s>>>(src, dst)); break;
    case 4: GB_LAUNCH("slice_digits", s, digits_blocked_kernel<4><<<grid, 256, 0, s>>>(src, dst)); break;
    case 5: GB_LAUNCH("slice_digits", s, digits_blocked_kernel<5><<<grid, 256, 0, s>>>(src, dst)); break;
    default: GB_LAUNCH("slice_digits", s, digits_blocked_kernel<6><<<grid, 256, 0, s>>>(src, dst)); break;
  }
  return GB_OK;
}

}  // namespace gb
