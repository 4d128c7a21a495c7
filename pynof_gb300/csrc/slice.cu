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

// Balanced base-128 digits of round(x 2^(7S - E)), pre-weighted: digit s as
// the FP32 bits of d 2^(-7 s) (|d| <= 128, exact in bf16, so the upper half of
// those bits is the bf16 pattern; the lower half is zero).  The 64-bit integer
// xi = H 2^(7 NL) + L (0 <= L < 2^(7 NL)) is taken apart in 32-bit pieces: the
// NL lowest digits come from L (its carry, 0 or 1, goes to H), the others from
// H.  Each digit's FP32 value comes from the 1.5 * 2^23 magic number (exact for
// |d| < 2^22), scaled by 2^(-7 s) in the same (exact) fused multiply-add.
template <int S>
__device__ __forceinline__ void make_digits(double x, int E, uint32_t* out) {
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
  constexpr int NL = S - 1 < 3 ? S - 1 : 3;
  int L = (int)(xi & ((1ll << (7 * NL)) - 1));
  int H = (int)(xi >> (7 * NL));
#pragma unroll
  for (int s = S; s > S - NL; --s) {
    const int d = ((L + 64) & 127) - 64;
    L = (L - d) >> 7;
    const float w = __int_as_float((127 - 7 * s) << 23);
    out[s - 1] = __float_as_uint(fmaf(__int_as_float(0x4B400000 + d), w, -12582912.0f * w));
  }
  H += L;
#pragma unroll
  for (int s = S - NL; s >= 2; --s) {
    const int d = ((H + 64) & 127) - 64;
    H = (H - d) >> 7;
    const float w = __int_as_float((127 - 7 * s) << 23);
    out[s - 1] = __float_as_uint(fmaf(__int_as_float(0x4B400000 + d), w, -12582912.0f * w));
  }
  const float w1 = __int_as_float((127 - 7) << 23);
  out[0] = __float_as_uint(fmaf(__int_as_float(0x4B400000 + H), w1, -12582912.0f * w1));
}

// A NaN or an infinity has the largest magnitude bits of all; it has no digits,
// so the row that holds one is reported in the status word (the first error
// recorded there stays) and the split-product kernels refuse to start.
__device__ __forceinline__ void note_nonfinite(unsigned long long maxbits, int* status) {
  if (maxbits >= 0x7FF0000000000000ull && status) atomicCAS(status, 0, GB_ERR_NONFINITE);
}

// One warp per row; K is the unit-stride index.
__global__ void rowexp_kfast_kernel(SliceSrc src, int rows, int K, int* __restrict__ exps, int* status) {
  const long long b = blockIdx.y;
  const long long row = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= rows) return;
  const double* base = src.p + b * src.sb + src.row_at(row);
  unsigned long long mx = 0;
  if (src.k.div == 0) {
    for (int k = lane; k < K; k += 32) {
      const unsigned long long v = abs_bits(base[(long long)k * src.k.s0]);
      mx = v > mx ? v : mx;
    }
  } else {
    // k runs of length div (stride s0 inside, s1 between runs): no division per element
    const long long div = src.k.div;
    for (long long k0 = 0, r = 0; k0 < K; k0 += div, ++r) {
      const double* bp = base + r * src.k.s1;
      const long long lim = K - k0 < div ? K - k0 : div;
      for (long long j = lane; j < lim; j += 32) {
        const unsigned long long v = abs_bits(bp[j * src.k.s0]);
        mx = v > mx ? v : mx;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = v > mx ? v : mx;
  }
  if (lane == 0) {
    exps[b * rows + row] = exponent_of(mx);
    note_nonfinite(mx, status);
  }
}

// Rows are the unit-stride index: 32 consecutive rows per CTA (lane = row,
// each warp reads 256 contiguous bytes per k) and its 8 warps split K; the
// partial maxima meet in shared memory.
__global__ void __launch_bounds__(256) rowexp_rfast_kernel(SliceSrc src, int rows, int K, int* __restrict__ exps,
                                                           int* status) {
  __shared__ unsigned long long part[8][32];
  const long long b = blockIdx.y;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long row = (long long)blockIdx.x * 32 + lane;
  unsigned long long mx = 0;
  if (row < rows) {
    const double* base = src.p + b * src.sb + src.row_at(row);
    for (int k = w; k < K; k += 8) {
      const unsigned long long v = abs_bits(base[src.k.at(k)]);
      mx = v > mx ? v : mx;
    }
  }
  part[w][lane] = mx;
  __syncthreads();
  if (w == 0 && row < rows) {
#pragma unroll
    for (int j = 1; j < 8; ++j) mx = part[j][lane] > mx ? part[j][lane] : mx;
    exps[b * rows + row] = exponent_of(mx);
    note_nonfinite(mx, status);
  }
}

// k blocks per CTA of the digit slicer
constexpr int SL_KPC = 8;

// The 8 source values of thread (row r, k group at k0) of one k block.
__device__ __forceinline__ void load_group(const SliceSrc& src, const double* base, bool rok, int k0, int K,
                                           double (&xs)[8]) {
  // k0 is a multiple of 8: with a unit k stride inside runs of a multiple of 8
  // (k.div), the 8 values are contiguous
  const double* p8 = base + src.k.at(k0);
  if (rok && src.kfast && src.k.s0 == 1 && (src.k.div == 0 || src.k.div % 8 == 0) && k0 + 8 <= K &&
      (reinterpret_cast<uintptr_t>(p8) & 15) == 0) {
    // contiguous, 16-byte aligned k run: four 16-byte loads
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const double2 v = __ldg(reinterpret_cast<const double2*>(p8) + u);
      xs[2 * u] = v.x;
      xs[2 * u + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int k = k0 + u;
      xs[u] = (rok && k < K) ? base[src.k.at(k)] : 0.0;
    }
  }
}

// Digits of the 8 values, packed per slice as 8 bf16 (one 16-byte store each).
template <int S>
__device__ __forceinline__ void store_group(const double (&xs)[8], int e, unsigned char* out) {
  uint32_t pk[S][4];
#pragma unroll
  for (int u = 0; u < 8; u += 2) {
    uint32_t d0[S], d1[S];
    make_digits<S>(xs[u], e, d0);
    make_digits<S>(xs[u + 1], e, d1);
    // the two bf16 patterns (upper halves) side by side
#pragma unroll
    for (int s = 0; s < S; ++s) pk[s][u >> 1] = __byte_perm(d0[s], d1[s], 0x7632);
  }
#pragma unroll
  for (int s = 0; s < S; ++s)
    *reinterpret_cast<uint4*>(out + (long long)s * SL_TILE_BYTES) = make_uint4(pk[s][0], pk[s][1], pk[s][2], pk[s][3]);
}

// One CTA of 256 threads per (row block, run of SL_KPC consecutive k blocks):
// thread -> (row r, k group of 8).  Lanes 0..7 take consecutive rows of one
// core matrix and a warp covers 32 consecutive rows of one k group, i.e. four
// whole consecutive core matrices (512 contiguous bytes) per slice, written
// with 16-byte stores; it reads 64 contiguous source bytes per row and k block
// (K-fast sources: the run reads SL_KPC x 128 contiguous bytes of each row) or
// 256 contiguous bytes per k (row-fast sources).  At most 64 registers (four
// CTAs per SM): occupancy keeps more loads in flight than prefetching the next
// k block into registers did (measured: 1.62 ms against 1.87-1.93 ms for the
// T of one nbf=600 build, 8.64 GB).
template <int S>
__global__ void __launch_bounds__(256, 4) digits_blocked_kernel(SliceSrc src, SlicedDesc dst) {
  const long long b = blockIdx.y;
  const int kbn = dst.kblocks();
  const int runs = (kbn + SL_KPC - 1) / SL_KPC;
  const int rb = blockIdx.x / runs, kb0 = (blockIdx.x % runs) * SL_KPC;
  const int kb1 = min(kb0 + SL_KPC, kbn);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ri = lane & 7, kg = warp >> 2, rg = (warp & 3) * 4 + (lane >> 3);
  const int r = rb * SL_ROWS + rg * 8 + ri;
  const bool rok = r < dst.rows;
  const double* base = src.p + b * src.sb + (rok ? src.row_at(r) : 0);
  const int e = rok ? dst.exps[b * dst.rows + r] : 0;
  unsigned char* out0 = reinterpret_cast<unsigned char*>(dst.planes) + b * dst.batch_bytes() +
                        ((long long)rb * kbn * S) * SL_TILE_BYTES + (kg * 16 + rg) * 128 + ri * 16;
  double xa[8];
  for (int kb = kb0; kb < kb1; ++kb) {
    load_group(src, base, rok, kb * SL_K + kg * 8, dst.K, xa);
    store_group<S>(xa, e, out0 + (long long)kb * S * SL_TILE_BYTES);
  }
}

// TF32 hi / lo of y = x 2^-E (|x| < 2^E), as FP32 bit patterns: hi = tf32(y),
// lo = tf32(y - hi), each rounded to nearest even to 11 significant bits from
// the FP64 bits with integer arithmetic (y - hi is exact); values below the
// FP32 normal range are flushed to zero.
__device__ __forceinline__ void tf32_split(double x, int E, uint32_t& hi, uint32_t& lo) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const uint32_t sign = (uint32_t)(bits >> 63);
  const int ex = (int)((bits >> 52) & 0x7FF);
  hi = 0u;
  lo = 0u;
  if (ex == 0) return;  // zero (FP64 subnormals are far below the FP32 range after scaling)
  const unsigned long long m = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);  // y = m 2^(ex - 1075 - E)
  int fe = ex - E - 1023 + 127;
  unsigned long long q = m >> 42;
  const unsigned long long rem = m & ((1ull << 42) - 1), half = 1ull << 41;
  if (rem > half || (rem == half && (q & 1ull))) ++q;
  const long long r = (long long)m - (long long)(q << 42);  // |r| <= 2^41
  if (q == (1ull << 11)) {
    q >>= 1;
    ++fe;
  }
  if (fe > 0) hi = (sign << 31) | ((uint32_t)fe << 23) | (((uint32_t)q & 0x3FFu) << 13);
  if (r == 0 || fe <= 0) return;
  const uint32_t rs = sign ^ (r < 0 ? 1u : 0u);
  const unsigned long long ra = (unsigned long long)(r < 0 ? -r : r);
  int top = 63 - __clzll((long long)ra);  // leading one of |r|
  unsigned long long q2;
  if (top > 10) {
    const int sh = top - 10;
    q2 = ra >> sh;
    const unsigned long long rem2 = ra & ((1ull << sh) - 1), h2 = 1ull << (sh - 1);
    if (rem2 > h2 || (rem2 == h2 && (q2 & 1ull))) ++q2;
    if (q2 == (1ull << 11)) {
      q2 >>= 1;
      ++top;
    }
  } else {
    q2 = ra << (10 - top);
  }
  const int fe2 = ex - 1075 - E + top + 127;
  if (fe2 > 0) lo = (rs << 31) | ((uint32_t)fe2 << 23) | (((uint32_t)q2 & 0x3FFu) << 13);
}

// TF32x3 planes, one CTA of 256 threads per (row block, k block of 8): thread
// -> (row r, k group of 4), 16-byte stores per plane (same thread map as the
// bf16 digits).
__global__ void __launch_bounds__(256) tf32_blocked_kernel(SliceSrc src, SlicedDesc dst) {
  const long long b = blockIdx.y;
  const int kbn = dst.kblocks();
  const int rb = blockIdx.x / kbn, kb = blockIdx.x % kbn;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ri = lane & 7, kg = warp >> 2, rg = (warp & 3) * 4 + (lane >> 3);
  const int r = rb * SL_ROWS + rg * 8 + ri;
  const int k0 = kb * (SL_K / 2) + kg * 4;
  const bool rok = r < dst.rows;
  const double* base = src.p + b * src.sb + (rok ? src.row_at(r) : 0);
  const int e = rok ? dst.exps[b * dst.rows + r] : 0;
  uint32_t hi[4], lo[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int k = k0 + u;
    tf32_split((rok && k < dst.K) ? base[src.k.at(k)] : 0.0, e, hi[u], lo[u]);
  }
  unsigned char* out = reinterpret_cast<unsigned char*>(dst.planes) + b * dst.batch_bytes() +
                       ((long long)blockIdx.x * 2) * SL_TILE_BYTES + (kg * 16 + rg) * 128 + ri * 16;
  *reinterpret_cast<uint4*>(out) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
  *reinterpret_cast<uint4*>(out + SL_TILE_BYTES) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
}

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

int slice_operand(const SliceSrc& src, const SlicedDesc& dst, cudaStream_t s, bool exps_ready) {
  GB_REQUIRE((dst.kind == 0 && dst.S >= 1 && dst.S <= 6) || (dst.kind == 1 && dst.S == 2), GB_ERR_INVALID_ARG,
             "slice_operand: bad split form (planes %d, kind %d)", dst.S, dst.kind);
  GB_REQUIRE(dst.batch >= 1 && dst.batch <= 65535 && dst.rows >= 0, GB_ERR_BAD_SHAPE, "slice_operand: bad batch");
  GB_REQUIRE((reinterpret_cast<uintptr_t>(dst.planes) & 15) == 0, GB_ERR_INVALID_ARG,
             "slice_operand: planes not 16-byte aligned");
  if (dst.rows == 0 || dst.K == 0) return GB_OK;
  if (exps_ready) {
    GB_REQUIRE(dst.kind == 0, GB_ERR_INVALID_ARG, "slice_operand: recorded exponents are for digit slices");
  } else if (src.kfast) {
    int* st = device_status_word();
    GB_LAUNCH("slice_rowexp", s,
              rowexp_kfast_kernel<<<dim3(cdiv(dst.rows, 8), dst.batch), 256, 0, s>>>(src, dst.rows, dst.K, dst.exps,
                                                                                    st));
  } else {
    int* st = device_status_word();
    GB_LAUNCH("slice_rowexp", s,
              rowexp_rfast_kernel<<<dim3(cdiv(dst.rows, 32), dst.batch), 256, 0, s>>>(src, dst.rows, dst.K,
                                                                                     dst.exps, st));
  }
  const long long blocks = (long long)dst.rblocks() * dst.kblocks();
  GB_REQUIRE(blocks <= 2147483647LL, GB_ERR_BAD_SHAPE, "slice_operand: too many blocks");
  if (dst.kind == 1) {
    GB_LAUNCH("slice_tf32", s, tf32_blocked_kernel<<<dim3((unsigned)blocks, dst.batch), 256, 0, s>>>(src, dst));
    return GB_OK;
  }
  const dim3 grid((unsigned)((long long)dst.rblocks() * ((dst.kblocks() + SL_KPC - 1) / SL_KPC)), dst.batch);
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
