// tcgen05 split-product FP64 GEMM (see ozaki_tc.cuh).
//
// CTA tile: 128 rows of A (M) x BN rows of B (N), BN in {32, 64, 128}.
// 18 warps.  warp 0 lane 0 is the producer: a 4-stage ring in which every
// stage holds the S slices of a 128 x 16 block of A (one contiguous
// cp.async.bulk copy -- the slicer stores the digits in the tensor-core
// core-matrix order, slice.cuh) and of a BN x 16 block of B (one copy, or two
// per slice when BN < 128).  warp 1 allocates TMEM (4 BN columns) and its
// lane 0 issues tcgen05.mma (M=128, N=BN, K=16, bf16 -> f32).  warps 2..17
// drain and finish: warp w reads TMEM lanes 32 (w % 4) .. +31 (tile rows) and
// BN/4 columns from (w - 2) / 4 * BN/4 of every accumulator.
//
// TMEM columns: [0,BN) group 2, [BN,2BN) group 3, [2BN,3BN) group 4 (exact,
// drained every 12 stages = 192 k), [3BN,4BN) groups 5.. (whole K, or per
// chunk with fdrain).
//
// One launch covers one GEMM (optionally batched), or -- the grouped kernel --
// a table of GEMMs of different shapes (e.g. one per molecule of a batch).
//
// Every mbarrier wait is bounded (the launch's wait_ns, 2 s unless
// gb_set_wait_limit_ns changed it); on timeout the CTA records GB_ERR_TIMEOUT
// in the device status word, stops issuing work, waits (bounded) for its own
// TMA copies and MMAs in flight, frees TMEM and exits.
#include <cuda_bf16.h>

#include <cuda.h>

#include <atomic>
#include <cstdio>
#include <mutex>
#include <vector>

#include "ozaki_tc.cuh"

static __device__ int g_tc_status;

namespace gb {
namespace {

constexpr int BM = 128, BK = SL_K, STAGES = 4, CH = 12;
constexpr int NUM_EPI_WARPS = 16, THREADS = 32 * (2 + NUM_EPI_WARPS);
// 18 warps put 5 warps on two of the four SM sub-partitions, whose register
// files hold 16K registers each: 5 * 32 * 96 <= 16384 caps the kernel at 96.
constexpr int MAX_REGS = 96;
constexpr uint32_t TILE_BYTES = SL_TILE_BYTES;  // 4 KB per A slice tile (BM == SL_ROWS)

// KIND 0: bf16 digit slices (kind::f16), four accumulators (three exact
// groups and the FP32 group); KIND 1: TF32x3 (kind::tf32), two FP32
// accumulators used alternately by consecutive chunks (one is drained while
// the MMAs fill the other).
template <int BN, int KIND>
struct TileCfg {
  static_assert(BN == 32 || BN == 64 || BN == 128, "BN must be 32, 64 or 128");
  static constexpr uint32_t B_TILE = BN * SL_K * 2;              // bytes of one B slice tile
  static constexpr uint32_t TMEM_COLS = KIND ? 2 * BN : 4 * BN;  // power of two >= 32
  static constexpr int CW = BN / 4;                              // columns per epilogue warp
  static constexpr int KPER = KIND ? SL_K / 2 : SL_K;            // k per stage (one MMA)
  static constexpr uint32_t FMT = KIND ? 2u : 1u;                // operand format: tf32 / bf16
  // instruction descriptor: f32 accumulate, both operands K-major, M=128, N=BN
  static constexpr uint32_t IDESC = (1u << 4) | (FMT << 7) | (FMT << 10) | ((uint32_t)(BN >> 3) << 17) |
                                    ((uint32_t)(BM >> 4) << 24);
};
// bytes of the per-tile assembly tables (see cta_tile)
__host__ __device__ constexpr uint32_t epi_table_bytes(int BN) { return 20u * (uint32_t)(BM + BN); }
constexpr float MAGIC = 12582912.0f;                          // 1.5 * 2^23
constexpr int MAGIC_BITS = 0x4B400000;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// Bounded wait: false after limit_ns, or (if abort_flag != nullptr) as soon
// as another role has aborted.
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag, unsigned long long limit_ns) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = now_ns();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try(bar, parity)) return true;
    if (abort_flag && *abort_flag) return false;
    if ((it & 63) == 0 && now_ns() - t0 > limit_ns) return false;
  }
}

// Named barrier of the 16 epilogue warps with an OR reduction: every one of
// them gets the same answer, so their control flow cannot diverge.
__device__ __forceinline__ bool epi_barrier_any(bool pred) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred pin, pout;\n setp.ne.u32 pin, %1, 0;\n"
      " bar.red.or.pred pout, 1, %2, pin;\n selp.u32 %0, 1, 0, pout;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)pred), "n"(NUM_EPI_WARPS * 32)
      : "memory");
  return r != 0;
}

// The first error recorded in the status word stays (a timeout does not
// overwrite an earlier non-finite report, nor the other way round).
__device__ __forceinline__ void signal_abort(volatile int* abort_flag) {
  *abort_flag = 1;
  atomicCAS(&g_tc_status, 0, GB_ERR_TIMEOUT);
}

// Contiguous global -> shared bulk copy completing on an mbarrier.
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// UMMA shared-memory descriptor of one slice tile of `rows` rows x 16 k:
// K-major, no swizzle; core matrices (8 rows x 16 B) rows*16 B apart along K
// (leading byte offset) and 128 B apart along the rows (stride byte offset).
__device__ __forceinline__ uint64_t desc_tile(uint32_t saddr, uint32_t rows) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((rows * 16u) >> 4) << 16;  // leading byte offset
  d |= (uint64_t)(128u >> 4) << 32;          // stride byte offset
  d |= (uint64_t)1 << 46;                    // descriptor version
  return d;                                  // layout type 0: no swizzle
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 8 consecutive TMEM columns of this warp's 32 lanes; complete after tmem_wait_ld().
__device__ __forceinline__ void tmem_ld8_async(uint32_t taddr, uint32_t (&v)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
               : "r"(taddr)
               : "memory");
}
__device__ __forceinline__ void tmem_ld4_async(uint32_t taddr, uint32_t (&v)[4]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
               : "r"(taddr)
               : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Exact integer of an FP32 value x * 2^k with |x * 2^k| < 2^22 (rounded to
// nearest even otherwise): adding 1.5 * 2^23 leaves the integer in the low
// mantissa bits.  Pure FP32/ALU work, no float->int conversion unit.
__device__ __forceinline__ int magic_int(float x, float scale) {
  return __float_as_int(fmaf(x, scale, MAGIC)) - MAGIC_BITS;
}

// t * 2^frac rounded to nearest as a 64-bit integer, for |t| < 2^22 and
// frac <= 16: rint(t) * 2^frac + rint((t - rint(t)) * 2^frac), both parts
// through magic_int; (t - rint(t)) is exact.
__device__ __forceinline__ long long split_round(float t, int frac, float two_frac) {
  const float f1 = t + MAGIC;
  const int ti = __float_as_int(f1) - MAGIC_BITS;
  const int fi = magic_int(t - (f1 - MAGIC), two_frac);
  return (long long)((unsigned long long)(long long)ti << frac) + fi;
}

// Drain of the exact groups g = 2..gE of CW columns of this warp's TMEM lanes
// into R: group g holds FP32 integer multiples of 2^-7g below 2^22 units, taken
// out with magic_int and combined as sum_g i_g 2^(7 (gE - g)) (units of
// 2^-7gE; groups 3 and 4 fit one int32, < 2^30), scaled by 2^fr.
template <int BN, int gE, int CW>
__device__ __forceinline__ void drain_exact(uint32_t lbase, long long (&R)[CW], int fr) {
#pragma unroll
  for (int h = 0; h < CW / 4; ++h) {
    uint32_t v2[4], v3[4], v4[4];
    tmem_ld4_async(lbase + (uint32_t)(h * 4), v2);
    if (gE >= 3) tmem_ld4_async(lbase + (uint32_t)(BN + h * 4), v3);
    if (gE >= 4) tmem_ld4_async(lbase + (uint32_t)(2 * BN + h * 4), v4);
    tmem_wait_ld();
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int i2 = magic_int(__uint_as_float(v2[j]), 16384.0f);  // 2^14
      long long acc;
      if (gE == 2) {
        acc = i2;
      } else if (gE == 3) {
        acc = (long long)i2 * 128 + magic_int(__uint_as_float(v3[j]), 2097152.0f);  // 2^21
      } else {
        const int i34 = magic_int(__uint_as_float(v3[j]), 2097152.0f) * 128 +
                        magic_int(__uint_as_float(v4[j]), 268435456.0f);  // 2^28
        acc = (long long)i2 * 16384 + i34;
      }
      R[h * 4 + j] += (long long)((unsigned long long)acc << fr);
    }
  }
}

// int64 fixed point z * 2^scale -> double, round to nearest even, integer ops
// only (the FP64 pipe is narrow on this part).  The leading one is moved to
// bit 63; the top 53 bits are the significand (implicit bit included, so adding
// it to (exponent - 1) << 52 forms the exponent field and a rounding carry out
// of the significand bumps the exponent), the low 11 bits decide the rounding.
__device__ __forceinline__ double fixed_to_double(long long z, int scale, int negate) {
  if (z == 0) return 0.0;
  const unsigned long long sign = (unsigned long long)((z < 0) != (negate != 0)) << 63;
  const unsigned long long u = z < 0 ? 0ull - (unsigned long long)z : (unsigned long long)z;
  const int lz = __clzll((long long)u);
  const unsigned long long m = u << lz;
  const unsigned long long mant = m >> 11;
  const uint32_t low = (uint32_t)m & 0x7FFu;
  const unsigned long long up = (low > 0x400u || (low == 0x400u && (mant & 1ull))) ? 1ull : 0ull;
  const int ef = 63 - lz + scale + 1023;  // biased exponent of the leading one
  if (ef <= 0) return __longlong_as_double((long long)sign);  // underflow -> signed zero
  if (ef >= 2047) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));
  return __longlong_as_double((long long)(sign | ((((unsigned long long)(ef - 1)) << 52) + mant + up)));
}

// z * 2^scale as a double, negated when `negate`: the hardware int64 -> double
// conversion (round to nearest even, as fixed_to_double) with the scale added
// to the exponent field; results outside the normal range take the integer path.
__device__ __forceinline__ double scaled_to_double(long long z, int scale, int negate) {
  const long long b0 = __double_as_longlong(__ll2double_rn(z));
  const int e0 = (int)((b0 >> 52) & 0x7FF) + scale;
  if (z != 0 && e0 >= 1 && e0 <= 2046)
    return __longlong_as_double((long long)(((unsigned long long)b0 + ((unsigned long long)(long long)scale << 52)) ^
                                            ((unsigned long long)(negate != 0) << 63)));
  return fixed_to_double(z, scale, negate);
}

struct KArgs {
  OzGemm g;
  SlicedDesc A, B;
  int frac;
  unsigned long long wait_ns;  // limit of every mbarrier wait
  // Test hook: the first CTA's producer never issues global stage `withhold`
  // (-1: every stage is issued), so the MMA issuer's wait for it runs out.
  int withhold;
};

// bf16 MMA with an A-collector qualifier: COLL 0 none, 1 fill (read A from
// shared memory and keep it in the tensor core's collector), 2 use (take A
// from the collector), 3 lastuse (take it and release the collector).
template <int COLL>
__device__ __forceinline__ void mma_bf16_c(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, bool accumulate) {
  if constexpr (COLL == 0)
    mma_bf16(d_tmem, a, b, idesc, accumulate);
  else if constexpr (COLL == 1)
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16.collector::a::fill [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)accumulate)
        : "memory");
  else if constexpr (COLL == 2)
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16.collector::a::use [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)accumulate)
        : "memory");
  else
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16.collector::a::lastuse [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)accumulate)
        : "memory");
}

// Products of one stage (S digit slices; product (s, t) of A slice s and B
// slice t goes to group g = s + t, kept only for g <= S + 1), fully unrolled
// and ordered by A slice: the products of one A slice run back to back and
// take A from the collector after the first, so each A slice tile is read
// from shared memory once per stage (6 reads instead of 21 at S = 6; B is
// read per product).  The slice tiles' descriptors differ from the stage's
// first ones only in the start-address field.
//   SEL 0: every product; 1: the FP32 group only (g >= 5); 2: the exact
//   groups only (g <= 4, accumulator columns (g - 2) BN).
//   restart_exact: the exact groups start from zero (their first product,
//   s = 1, overwrites); restart_f: the FP32 group (at 3 BN) starts from zero.
template <int S, int BN, int SEL>
__device__ __forceinline__ void issue_products(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc,
                                               bool restart_exact, bool restart_f) {
  using T = TileCfg<BN, 0>;
  bool f_first = true;
#pragma unroll
  for (int s = 1; s <= S; ++s) {
    const uint64_t das = da + (uint64_t)((s - 1) * (TILE_BYTES >> 4));
    // this slice's products under SEL: t in [t0, t1]
    const int t0 = SEL == 1 ? (5 - s > 1 ? 5 - s : 1) : 1;
    const int t1 = SEL == 2 ? (4 - s < S + 1 - s ? 4 - s : S + 1 - s) : S + 1 - s;
#pragma unroll
    for (int t = t0; t <= t1; ++t) {
      const int gg = s + t;
      const bool exact = gg <= 4;
      const uint32_t d = tmem + (uint32_t)((exact ? gg - 2 : 3) * BN);
      const uint64_t dbt = db + (uint64_t)((t - 1) * (T::B_TILE >> 4));
      bool acc;
      if (exact) {
        acc = !(restart_exact && s == 1);
      } else {
        acc = !(restart_f && f_first);
        f_first = false;
      }
      if (t0 == t1)
        mma_bf16_c<0>(d, das, dbt, idesc, acc);
      else if (t == t0)
        mma_bf16_c<1>(d, das, dbt, idesc, acc);
      else if (t == t1)
        mma_bf16_c<3>(d, das, dbt, idesc, acc);
      else
        mma_bf16_c<2>(d, das, dbt, idesc, acc);
    }
  }
}

// TF32x3 products of one stage: hi hi + hi lo + lo hi into the one accumulator.
template <int BN>
__device__ __forceinline__ void issue_tf32(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, bool& started) {
  using T = TileCfg<BN, 1>;
  mma_tf32(tmem, da, db, idesc, started);
  mma_tf32(tmem, da, db + (uint64_t)(T::B_TILE >> 4), idesc, true);
  mma_tf32(tmem, da + (uint64_t)(TILE_BYTES >> 4), db, idesc, true);
  started = true;
}

// Problem of global tile u in a grouped launch: the p with starts[p] <= u <
// starts[p + 1] (always 0 for a single problem, starts == nullptr).
__device__ __forceinline__ int find_problem(const long long* starts, int nprob, unsigned int u) {
  if (starts == nullptr || nprob <= 1) return 0;
  int lo = 0, hi = nprob;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (starts[mid] <= (long long)u) lo = mid; else hi = mid;
  }
  return lo;
}

// The problem a tile belongs to: the table entry of a grouped launch, the
// launch's own argument otherwise.
template <bool GROUPED>
__device__ __forceinline__ const KArgs& prob_ref(const KArgs& a0, const KArgs* probs, int p) {
  if constexpr (GROUPED) return probs[p];
  else return a0;
}

// Local tile index -> (batch, m0, n0).  The dimension with fewer tiles runs
// fastest, so that the CTAs sharing a block of the large operand run together
// (that block is read once from HBM, then from L2).  Returns false
// for tiles a symmetric output does not need.
template <int BN>
__device__ __forceinline__ bool decode_tile(const OzGemm& g, long long t, int& bz, int& m0, int& n0) {
  const int mtiles = (g.M + BM - 1) / BM;
  const int ntiles = (g.N + BN - 1) / BN;
  const long long per_batch = (long long)mtiles * ntiles;
  bz = (int)(t / per_batch);
  const long long r = t % per_batch;
  if (mtiles <= ntiles) {
    m0 = (int)(r % mtiles) * BM;
    n0 = (int)(r / mtiles) * BN;
  } else {
    n0 = (int)(r % ntiles) * BN;
    m0 = (int)(r / ntiles) * BM;
  }
  return !(g.sym == SYM_ROWCOL && m0 > n0);
}

// One output tile, all roles.
template <int S, int BN, int KIND>
__device__ __forceinline__ void cta_tile(const KArgs& a, int bz, int m0, int n0, unsigned char* smem_raw) {
  using T = TileCfg<BN, KIND>;
  const OzGemm& g = a.g;
  constexpr int gE = (S + 1) < 4 ? (S + 1) : 4;
  constexpr bool has_inexact = (S + 1) > 4;
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  constexpr uint32_t a_bytes = (uint32_t)S * TILE_BYTES, b_bytes = (uint32_t)S * T::B_TILE;
  constexpr uint32_t stage_bytes = a_bytes + b_bytes;
  // the assembly parks the tile's int64 results in the stage buffers
  constexpr uint32_t zs_bytes = BM * (BN + 1) * 8;
  constexpr uint32_t data_bytes = STAGES * stage_bytes > zs_bytes ? STAGES * stage_bytes : zs_bytes;
  // assembly tables: roff, mr [BM], coff, mc [BN] (int64), srow [BM], scol [BN] (int)
  long long* e_roff = reinterpret_cast<long long*>(smem + data_bytes);
  long long* e_mr = e_roff + BM;
  long long* e_coff = e_mr + BM;
  long long* e_mc = e_coff + BN;
  int* e_srow = reinterpret_cast<int*>(e_mc + BN);
  int* e_scol = e_srow + BM;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + data_bytes + epi_table_bytes(BN));
  // bars: full[STAGES], empty[STAGES], accfull, accempty, done, (slot, flag), accfull1, accempty1
  volatile uint32_t* tmem_slot = reinterpret_cast<volatile uint32_t*>(bars + 2 * STAGES + 4);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 2 * STAGES + 5);
  const uint32_t sbase = smem_u32(smem);
  const uint32_t bar0 = smem_u32(bars);
  auto full_bar = [&](int st) { return bar0 + 8u * st; };
  auto empty_bar = [&](int st) { return bar0 + 8u * (STAGES + st); };
  const uint32_t accfull_bar = bar0 + 8u * (2 * STAGES), accempty_bar = bar0 + 8u * (2 * STAGES + 1),
                 done_bar = bar0 + 8u * (2 * STAGES + 2);
  // TF32x3: the second accumulator's pair (chunk c uses accumulator c & 1)
  const uint32_t accfull1_bar = bar0 + 8u * (2 * STAGES + 6), accempty1_bar = bar0 + 8u * (2 * STAGES + 7);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(full_bar(i), 1);
      mbar_init(empty_bar(i), 1);
    }
    mbar_init(accfull_bar, 1);
    mbar_init(accempty_bar, NUM_EPI_WARPS);
    mbar_init(done_bar, 1);
    mbar_init(accfull1_bar, 1);
    mbar_init(accempty1_bar, NUM_EPI_WARPS);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(const_cast<uint32_t*>(tmem_slot))),
                 "r"(T::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    tc_fence_before();
  }
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  const int nkb = (g.K + T::KPER - 1) / T::KPER;
  const int nchunks = (nkb + CH - 1) / CH;
  // A ragged last column tile runs its MMAs only as wide as it needs (N a
  // multiple of 16 for M = 128); the idle epilogue warps skip their columns.
  const int n_valid = min(BN, g.N - n0);
  const int n_mma = (n_valid + 15) & ~15;
  const uint32_t idesc = (T::IDESC & ~(0x3Fu << 17)) | ((uint32_t)(n_mma >> 3) << 17);

  int issued = 0;  // stages the producer handled (its lane 0)
  if (warp == 0) {
    // ---------------- producer ----------------
    if (lane == 0) {
      // an operand sliced once (batch 1) is shared by every batch entry
      const long long abz = a.A.batch == 1 ? 0 : bz, bbz = a.B.batch == 1 ? 0 : bz;
      const unsigned char* ga = reinterpret_cast<const unsigned char*>(a.A.planes) + abz * a.A.batch_bytes() +
                                (long long)(m0 / BM) * a.A.kblocks() * a_bytes;
      const int rb = n0 / SL_ROWS, r0 = n0 % SL_ROWS;
      const unsigned char* gbp = reinterpret_cast<const unsigned char*>(a.B.planes) + bbz * a.B.batch_bytes() +
                                 (long long)rb * a.B.kblocks() * (S * TILE_BYTES) + (r0 / 8) * 128;
      for (int kb = 0; kb < nkb; ++kb) {
        const int st = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!mbar_wait(empty_bar(st), ph ^ 1, abort_flag, a.wait_ns)) {
          signal_abort(abort_flag);
          break;
        }
        if (kb == a.withhold && blockIdx.x == 0 && blockIdx.y == 0) {
          ++issued;  // test hook: this stage never arrives
          continue;
        }
        mbar_expect_tx(full_bar(st), stage_bytes);
        const uint32_t sa = sbase + st * stage_bytes;
        bulk_load(sa, ga + (long long)kb * a_bytes, a_bytes, full_bar(st));
        const unsigned char* gblk = gbp + (long long)kb * (S * TILE_BYTES);
        if (BN == SL_ROWS) {
          bulk_load(sa + a_bytes, gblk, b_bytes, full_bar(st));
        } else {
          // BN rows of each k group of each slice tile: two runs of BN * 16 bytes
#pragma unroll
          for (int s = 0; s < S; ++s)
#pragma unroll
            for (int kg = 0; kg < 2; ++kg)
              bulk_load(sa + a_bytes + s * T::B_TILE + kg * (BN * 16), gblk + s * TILE_BYTES + kg * 2048, BN * 16,
                        full_bar(st));
        }
        ++issued;
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      bool f_started = false;
      for (int kb = 0; kb < nkb; ++kb) {
        const int st = kb % STAGES;
        if (!mbar_wait(full_bar(st), (kb / STAGES) & 1, abort_flag, a.wait_ns)) {
          signal_abort(abort_flag);
          break;
        }
        tc_fence_after();
        const uint32_t sa = sbase + st * stage_bytes;
        const uint64_t da = desc_tile(sa, BM), db = desc_tile(sa + a_bytes, BN);
        if constexpr (KIND == 1) {
          // chunk c accumulates in buffer c & 1, drained by the epilogue while
          // chunk c + 1 runs; before reusing a buffer wait for its last drain
          const int c = kb / CH, bsel = c & 1;
          if ((kb % CH) == 0) {
            if (c >= 2) {
              if (!mbar_wait(bsel ? accempty1_bar : accempty_bar, ((c >> 1) - 1) & 1, abort_flag, a.wait_ns)) {
                signal_abort(abort_flag);
                break;
              }
              tc_fence_after();
            }
            f_started = false;
          }
          issue_tf32<BN>(tmem + (uint32_t)(bsel * BN), da, db, idesc, f_started);
          if ((kb % CH) == CH - 1 || kb == nkb - 1) mma_commit(bsel ? accfull1_bar : accfull_bar);
          mma_commit(empty_bar(st));
          continue;
        }
        const int c = kb / CH;
        const bool first = (kb % CH) == 0;
        if (!first) {
          issue_products<S, BN, 0>(tmem, da, db, idesc, false, false);
        } else if (c == 0) {
          issue_products<S, BN, 0>(tmem, da, db, idesc, true, true);
        } else if (g.fdrain) {
          // the FP32 accumulator is drained with the exact groups: it restarts
          // every chunk, after the drain
          if (!mbar_wait(accempty_bar, (c - 1) & 1, abort_flag, a.wait_ns)) {
            signal_abort(abort_flag);
            break;
          }
          tc_fence_after();
          issue_products<S, BN, 0>(tmem, da, db, idesc, true, true);
        } else {
          // the FP32 group runs ahead while the exact groups drain
          issue_products<S, BN, 1>(tmem, da, db, idesc, false, false);
          if (!mbar_wait(accempty_bar, (c - 1) & 1, abort_flag, a.wait_ns)) {
            signal_abort(abort_flag);
            break;
          }
          tc_fence_after();
          issue_products<S, BN, 2>(tmem, da, db, idesc, true, false);
        }
        if ((kb % CH) == CH - 1 || kb == nkb - 1) mma_commit(accfull_bar);
        mma_commit(empty_bar(st));
      }
      mma_commit(done_bar);
    }
  } else {
    // ---------------- epilogue: drain exact groups, assemble FP64 ----------------
    constexpr int CW = T::CW;
    const int q = warp & 3;
    const int cg = (warp - 2) >> 2;
    const int et = threadIdx.x - 64;  // 0 .. 511
    const uint32_t lbase = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(cg * CW);
    const bool cols_live = cg * CW < n_valid;  // warp-uniform
    // Row / column tables of the tile for the assembly, filled while the MMAs
    // run: output offsets, mirror offsets (-1: none) and exponent scales.
    {
      const long long abz = a.A.batch == 1 ? 0 : bz, bbz = a.B.batch == 1 ? 0 : bz;
      if (et < BM) {
        const int i = m0 + et;
        const bool in = i < g.M;
        long long mr = -1;
        if (in && g.sym == SYM_ROWCOL) mr = g.c_c.at(i);
        long long ri = i;  // the pair's index for a packed-triangle row
        if (in && g.sym == SYM_TRIROW) {
          int mm, nn;
          tri_pair(i, g.pair_n, mm, nn);
          ri = (long long)mm * g.pair_n + nn;
          if (nn > mm) mr = g.c_r.at((long long)nn * g.pair_n + mm);
        }
        e_roff[et] = in ? g.c_r.at(ri) : 0;
        e_mr[et] = mr;
        e_srow[et] = in ? a.A.exps[abz * g.M + i] : 0;
      } else if (et < BM + BN) {
        const int c = et - BM, jj = n0 + c;
        const bool in = jj < g.N;
        long long mc = -1;
        if (in && g.sym == SYM_ROWCOL) mc = g.c_r.at(jj);
        long long cj = jj;
        if (in && g.sym == SYM_TRICOL) {
          int mm, nn;
          tri_pair(jj, g.pair_n, mm, nn);
          cj = (long long)mm * g.pair_n + nn;
          if (nn > mm) mc = g.c_c.at((long long)nn * g.pair_n + mm);
        }
        e_coff[c] = in ? g.c_c.at(cj) : 0;
        e_mc[c] = mc;
        e_scol[c] = in ? a.B.exps[bbz * g.N + jj] - (KIND ? 31 : 7 * gE + a.frac) : 0;
      }
    }
    long long R[CW];
#pragma unroll
    for (int j = 0; j < CW; ++j) R[j] = 0;
    const float two_frac = __int_as_float((127 + a.frac) << 23);  // 2^frac
    const float upE = __int_as_float((127 + 7 * gE) << 23);       // 2^(7 gE)
    bool ok = true;
    for (int c = 0; c < nchunks; ++c) {
      if constexpr (KIND == 1) {
        // R (units of 2^-31) += rint(F 2^31): |F| < 2^7 per chunk of 96 k
        // (every |tf32 operand| < 1), so F 2^15 < 2^22 suits split_round
        const int bsel = c & 1;
        const bool got = mbar_wait(bsel ? accfull1_bar : accfull_bar, (c >> 1) & 1, abort_flag, a.wait_ns);
        if (!__all_sync(0xffffffffu, got)) {
          signal_abort(abort_flag);
          ok = false;
          break;
        }
        tc_fence_after();
        if (cols_live) {
#pragma unroll
          for (int h = 0; h < CW / 8; ++h) {
            uint32_t v[8];
            tmem_ld8_async(lbase + (uint32_t)(bsel * BN + h * 8), v);
            tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 8; ++j) R[h * 8 + j] += split_round(__uint_as_float(v[j]) * 32768.0f, 16, 65536.0f);
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(bsel ? accempty1_bar : accempty_bar);
        continue;
      }
      const bool got = mbar_wait(accfull_bar, c & 1, abort_flag, a.wait_ns);
      if (!__all_sync(0xffffffffu, got)) {
        signal_abort(abort_flag);
        ok = false;
        break;
      }
      tc_fence_after();
      const int fr = g.fdrain ? a.frac : 0;  // fraction bits carried by R from the start
      if (cols_live) drain_exact<BN, gE, CW>(lbase, R, fr);
      if (has_inexact && g.fdrain && cols_live) {
#pragma unroll
        for (int h = 0; h < CW / 8; ++h) {
          uint32_t v[8];
          tmem_ld8_async(lbase + (uint32_t)(3 * BN + h * 8), v);
          tmem_wait_ld();
#pragma unroll
          for (int j = 0; j < 8; ++j) R[h * 8 + j] += split_round(__uint_as_float(v[j]) * upE, a.frac, two_frac);
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(accempty_bar);
    }
    if (ok) {
      const bool got = mbar_wait(done_bar, 0, abort_flag, a.wait_ns);
      if (!__all_sync(0xffffffffu, got)) signal_abort(abort_flag);
    }

    // CTA-uniform go / no-go for the assembly (every epilogue warp arrives here)
    if (epi_barrier_any(*abort_flag != 0)) ok = false;
    if (ok) {
      tc_fence_after();
      double* Cb = g.C + (long long)bz * g.c_sb;
      const bool mirror_rc = (g.sym == SYM_ROWCOL) && (m0 != n0);
      const bool rows_fast = g.c_c.div == 0 && g.c_c.s0 == 1 ? false : (g.c_r.div == 0 && g.c_r.s0 == 1);
      const int rlim = min(BM, g.M - m0), clim = min(BN, g.N - n0);
      // one output element: convert and store (plus its mirror)
      auto put = [&](long long z, int scale, long long ro, long long co, long long mr, long long mc) {
        const double val = scaled_to_double(z, scale, g.negate);
        Cb[ro + co] = val;
        if (mirror_rc) {
          Cb[mc + mr] = val;
        } else if (g.sym == SYM_TRICOL) {
          if (mc >= 0) Cb[ro + mc] = val;
        } else if (g.sym == SYM_TRIROW) {
          if (mr >= 0) Cb[mr + co] = val;
        }
      };
      // 1) fold the FP32 accumulator into the fixed point.  When the output's
      //    unit-stride index is the tile row (the TMEM lane), this layout
      //    already stores coalesced: convert and store here.  Otherwise park z
      //    in shared memory (the stage buffers are idle once every MMA has
      //    completed) for a transposed pass.
      const int row = q * 32 + lane;
      long long* Zs = reinterpret_cast<long long*>(smem);
      // z of this thread's row for its CW columns, handed to sink(c, z)
      auto fold = [&](auto&& sink) {
#pragma unroll
        for (int h = 0; h < CW / 8; ++h) {
          if constexpr (KIND == 1) {
            // every chunk is already in R (fixed point, 31 fraction bits)
#pragma unroll
            for (int j = 0; j < 8; ++j) sink(cg * CW + h * 8 + j, R[h * 8 + j]);
          } else {
            uint32_t v[8];
            if (has_inexact && !g.fdrain && cols_live) {
              tmem_ld8_async(lbase + (uint32_t)(3 * BN + h * 8), v);
              tmem_wait_ld();
            } else {
#pragma unroll
              for (int j = 0; j < 8; ++j) v[j] = 0u;
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              long long z = R[h * 8 + j];
              if (!g.fdrain)
                z = (long long)((unsigned long long)z << a.frac) +
                    split_round(__uint_as_float(v[j]) * upE, a.frac, two_frac);
              sink(cg * CW + h * 8 + j, z);
            }
          }
        }
      };
      // (the TMEM loads inside fold are warp-collective: no per-thread branch around it)
      if (rows_fast) {
        const bool row_live = row < rlim;
        fold([&](int c, long long z) {
          if (row_live && c < clim) put(z, e_srow[row] + e_scol[c], e_roff[row], e_coff[c], e_mr[row], e_mc[c]);
        });
      } else {
        fold([&](int c, long long z) { Zs[row * (BN + 1) + c] = z; });
      }
      // 2) rows are not the unit stride: assemble FP64 from shared memory with
      //    each thread on one column, lanes along the columns
      constexpr int U = 4;  // elements in flight per thread
      if (!rows_fast) {
        epi_barrier_any(false);
        constexpr int RSTEP = NUM_EPI_WARPS * 32 / BN;
        constexpr int NIT = BM / RSTEP;
        const int c = et % BN, r0 = et / BN;
        if (c < clim) {
          const int sc = e_scol[c];
          const long long co = e_coff[c], mc = e_mc[c];
          if (rlim == BM) {
#pragma unroll 1
            for (int it = 0; it < NIT; it += U) {
              long long zv[U], ro[U], mr[U];
              int sr[U];
#pragma unroll
              for (int u = 0; u < U; ++u) {
                const int r = r0 + (it + u) * RSTEP;
                zv[u] = Zs[r * (BN + 1) + c];
                sr[u] = e_srow[r];
                ro[u] = e_roff[r];
                mr[u] = g.sym == SYM_NONE ? -1 : e_mr[r];
              }
#pragma unroll
              for (int u = 0; u < U; ++u) put(zv[u], sr[u] + sc, ro[u], co, mr[u], mc);
            }
          } else {
            for (int r = r0; r < rlim; r += RSTEP)
              put(Zs[r * (BN + 1) + c], e_srow[r] + sc, e_roff[r], co, e_mr[r], mc);
          }
        }
      }
    }
  }

  __syncthreads();
  // the abort flag is final here: after an abort, the copies the producer
  // issued must land before the CTA exits (a withheld stage's wait runs out)
  if (warp == 0 && lane == 0 && *abort_flag) {
    for (int kb = max(0, issued - STAGES); kb < issued; ++kb)
      mbar_wait(full_bar(kb % STAGES), (kb / STAGES) & 1, nullptr, a.wait_ns);
  }
  if (warp == 1) {
    if (*abort_flag) {
      // every MMA this CTA issued must be complete before TMEM is released
      mbar_wait(done_bar, 0, nullptr, a.wait_ns);
    }
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(T::TMEM_COLS) : "memory");
  }
}

// Persistent form (bf16 digits; outputs whose tile rows are the unit stride,
// so the epilogue stores straight from registers and never parks results in
// the stage buffers).  One CTA per SM; its producer takes the tiles from a
// counter in the caller's memory (so tiles start in order across the GPU, as
// with the hardware's block dispatch, and the CTAs that share a block of the
// large operand read it together) or, without one, walks t = blockIdx.x,
// + gridDim.x, ...; it hands each tile index to the MMA issuer and the
// epilogue through a small ring in shared memory.  The producer runs ahead across tile boundaries (the next
// tile's first stages load during this tile's epilogue), and the epilogue
// releases TMEM as soon as the last chunk is folded into registers, so the
// next tile's MMAs overlap the conversion and stores.  Pipeline phases
// (stages, chunks) count on across tiles.
template <int S, int BN, bool GROUPED>
__device__ __forceinline__ void cta_persistent(const KArgs& a0, const KArgs* __restrict__ probs,
                                               const long long* __restrict__ starts, int nprob, int ntiles,
                                               unsigned int* counter, unsigned char* smem_raw) {
  using T = TileCfg<BN, 0>;
  constexpr int gE = (S + 1) < 4 ? (S + 1) : 4;
  constexpr bool has_inexact = (S + 1) > 4;
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  constexpr uint32_t a_bytes = (uint32_t)S * TILE_BYTES, b_bytes = (uint32_t)S * T::B_TILE;
  constexpr uint32_t stage_bytes = a_bytes + b_bytes;
  constexpr uint32_t zs_bytes = BM * (BN + 1) * 8;  // same layout as cta_tile (smem_bytes)
  constexpr uint32_t data_bytes = STAGES * stage_bytes > zs_bytes ? STAGES * stage_bytes : zs_bytes;
  long long* e_roff = reinterpret_cast<long long*>(smem + data_bytes);
  long long* e_mr = e_roff + BM;
  long long* e_coff = e_mr + BM;
  long long* e_mc = e_coff + BN;
  int* e_srow = reinterpret_cast<int*>(e_mc + BN);
  int* e_scol = e_srow + BM;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + data_bytes + epi_table_bytes(BN));
  volatile uint32_t* tmem_slot = reinterpret_cast<volatile uint32_t*>(bars + 2 * STAGES + 4);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 2 * STAGES + 5);
  // tile hand-off from the producer to the MMA issuer and the epilogue: a
  // ring of (problem, tile) indices (tile -1 ends the walk) behind full /
  // empty barriers
  constexpr int RING = 4;
  static_assert(2 * STAGES + 6 <= 16 && (24 + RING) * 8 <= 256, "barrier block of smem_bytes");
  volatile int* ring = reinterpret_cast<volatile int*>(bars + 24);
  volatile int* ringp = ring + RING;
  const uint32_t ringbar0 = smem_u32(bars + 16);
  auto ring_full = [&](int r) { return ringbar0 + 8u * r; };
  auto ring_empty = [&](int r) { return ringbar0 + 8u * (RING + r); };
  const uint32_t sbase = smem_u32(smem);
  const uint32_t bar0 = smem_u32(bars);
  auto full_bar = [&](int st) { return bar0 + 8u * st; };
  auto empty_bar = [&](int st) { return bar0 + 8u * (STAGES + st); };
  const uint32_t accfull_bar = bar0 + 8u * (2 * STAGES), accempty_bar = bar0 + 8u * (2 * STAGES + 1),
                 done_bar = bar0 + 8u * (2 * STAGES + 2);
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(full_bar(i), 1);
      mbar_init(empty_bar(i), 1);
    }
    mbar_init(accfull_bar, 1);
    mbar_init(accempty_bar, NUM_EPI_WARPS);
    mbar_init(done_bar, 1);
    for (int r = 0; r < RING; ++r) {
      mbar_init(ring_full(r), 1);
      mbar_init(ring_empty(r), 1 + NUM_EPI_WARPS);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(const_cast<uint32_t*>(tmem_slot))),
                 "r"(T::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    tc_fence_before();
  }
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  int gkb_issued = 0;  // stages the producer handled, all tiles (its lane 0)
  if (warp == 0) {
    // ---------------- producer ----------------
    if (lane == 0) {
      int& gkb = gkb_issued;
      bool aborted = false;
      unsigned int next = blockIdx.x;  // static walk when no tile counter is given
      for (int i = 0; !aborted; ++i) {
        const int slot = i % RING;
        if (!mbar_wait(ring_empty(slot), (uint32_t)(((i / RING) & 1) ^ 1), abort_flag, a0.wait_ns)) {
          signal_abort(abort_flag);
          break;
        }
        // next tile that has work (tiles a symmetry skips are passed over here)
        int t, p = 0, bz, m0, n0;
        for (;;) {
          unsigned int u;
          if (counter) {
            u = atomicAdd(counter, 1u);
          } else {
            u = next;
            next += gridDim.x;
          }
          if (u >= (unsigned int)ntiles) {
            t = -1;
            break;
          }
          if constexpr (GROUPED) {
            p = find_problem(starts, nprob, u);
            t = (int)(u - starts[p]);
          } else {
            t = (int)u;
          }
          if (decode_tile<BN>(prob_ref<GROUPED>(a0, probs, p).g, t, bz, m0, n0)) break;
        }
        ring[slot] = t;
        ringp[slot] = p;
        mbar_arrive(ring_full(slot));
        if (t < 0) break;
        const KArgs& a = prob_ref<GROUPED>(a0, probs, p);
        const int nkb = (a.g.K + BK - 1) / BK;
        const long long abz = a.A.batch == 1 ? 0 : bz, bbz = a.B.batch == 1 ? 0 : bz;
        const unsigned char* ga = reinterpret_cast<const unsigned char*>(a.A.planes) + abz * a.A.batch_bytes() +
                                  (long long)(m0 / BM) * a.A.kblocks() * a_bytes;
        const int rb = n0 / SL_ROWS, r0 = n0 % SL_ROWS;
        const unsigned char* gbp = reinterpret_cast<const unsigned char*>(a.B.planes) + bbz * a.B.batch_bytes() +
                                   (long long)rb * a.B.kblocks() * (S * TILE_BYTES) + (r0 / 8) * 128;
        for (int kb = 0; kb < nkb; ++kb) {
          const int st = gkb % STAGES;
          const uint32_t ph = (uint32_t)((gkb / STAGES) & 1);
          if (!mbar_wait(empty_bar(st), ph ^ 1, abort_flag, a0.wait_ns)) {
            signal_abort(abort_flag);
            aborted = true;
            break;
          }
          if (gkb == a0.withhold && blockIdx.x == 0) {
            ++gkb;  // test hook: this stage never arrives
            continue;
          }
          mbar_expect_tx(full_bar(st), stage_bytes);
          const uint32_t sa = sbase + st * stage_bytes;
          bulk_load(sa, ga + (long long)kb * a_bytes, a_bytes, full_bar(st));
          const unsigned char* gblk = gbp + (long long)kb * (S * TILE_BYTES);
          if (BN == SL_ROWS) {
            bulk_load(sa + a_bytes, gblk, b_bytes, full_bar(st));
          } else {
#pragma unroll
            for (int s2 = 0; s2 < S; ++s2)
#pragma unroll
              for (int kg = 0; kg < 2; ++kg)
                bulk_load(sa + a_bytes + s2 * T::B_TILE + kg * (BN * 16), gblk + s2 * TILE_BYTES + kg * 2048, BN * 16,
                          full_bar(st));
          }
          ++gkb;
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int gkb = 0, gch = 0;
      bool aborted = false;
      for (int i = 0; !aborted; ++i) {
        const int slot = i % RING;
        if (!mbar_wait(ring_full(slot), (uint32_t)((i / RING) & 1), abort_flag, a0.wait_ns)) {
          signal_abort(abort_flag);
          break;
        }
        const int t = ring[slot], p = ringp[slot];
        mbar_arrive(ring_empty(slot));
        if (t < 0) break;
        const OzGemm& g = prob_ref<GROUPED>(a0, probs, p).g;
        const int nkb = (g.K + BK - 1) / BK;
        int bz, m0, n0;
        decode_tile<BN>(g, t, bz, m0, n0);
        const int n_valid = min(BN, g.N - n0);
        const int n_mma = (n_valid + 15) & ~15;
        const uint32_t idesc = (T::IDESC & ~(0x3Fu << 17)) | ((uint32_t)(n_mma >> 3) << 17);
        for (int kb = 0; kb < nkb; ++kb) {
          const int st = gkb % STAGES;
          if (!mbar_wait(full_bar(st), (uint32_t)((gkb / STAGES) & 1), abort_flag, a0.wait_ns)) {
            signal_abort(abort_flag);
            aborted = true;
            break;
          }
          tc_fence_after();
          const uint32_t sa = sbase + st * stage_bytes;
          const uint64_t da = desc_tile(sa, BM), db = desc_tile(sa + a_bytes, BN);
          const int c = kb / CH;
          const bool first = (kb % CH) == 0;
          const bool chunk_last = (kb % CH) == CH - 1 || kb == nkb - 1;
          // a new tile (or, with fdrain, every chunk) must wait until the
          // epilogue has taken everything out of TMEM; inside a tile the FP32
          // group may run ahead while the exact groups drain
          if (first && gch > 0 && (c == 0 || g.fdrain)) {
            if (!mbar_wait(accempty_bar, (uint32_t)((gch - 1) & 1), abort_flag, a0.wait_ns)) {
              signal_abort(abort_flag);
              aborted = true;
              break;
            }
            tc_fence_after();
          }
          if (first && c > 0 && !g.fdrain) {
            // the FP32 group runs ahead while the exact groups drain
            issue_products<S, BN, 1>(tmem, da, db, idesc, false, false);
            if (!mbar_wait(accempty_bar, (uint32_t)((gch - 1) & 1), abort_flag, a0.wait_ns)) {
              signal_abort(abort_flag);
              aborted = true;
              break;
            }
            tc_fence_after();
            issue_products<S, BN, 2>(tmem, da, db, idesc, true, false);
          } else {
            // the tile's first stage restarts every accumulator (with fdrain,
            // every chunk's first stage does)
            issue_products<S, BN, 0>(tmem, da, db, idesc, first, first && (c == 0 || g.fdrain));
          }
          mma_commit(empty_bar(st));
          if (chunk_last) {
            mma_commit(accfull_bar);
            ++gch;
          }
          ++gkb;
        }
      }
      mma_commit(done_bar);
    }
  } else {
    // ---------------- epilogue ----------------
    constexpr int CW = T::CW;
    const int q = warp & 3;
    const int cg = (warp - 2) >> 2;
    const int et = threadIdx.x - 64;
    const uint32_t lbase = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(cg * CW);
    const float upE = __int_as_float((127 + 7 * gE) << 23);
    const int row = q * 32 + lane;
    int gch = 0;
    for (int i = 0;; ++i) {
      const int slot = i % RING;
      const bool got = mbar_wait(ring_full(slot), (uint32_t)((i / RING) & 1), abort_flag, a0.wait_ns);
      if (!got) signal_abort(abort_flag);
      const int t = got ? ring[slot] : -1;
      const int p = got ? ringp[slot] : 0;
      __syncwarp();
      if (lane == 0) mbar_arrive(ring_empty(slot));
      // every epilogue warp is done with the previous tile's tables, and all
      // of them take the same branch
      if (epi_barrier_any(!got || *abort_flag != 0)) break;
      if (t < 0) break;
      const KArgs& a = prob_ref<GROUPED>(a0, probs, p);
      const OzGemm& g = a.g;
      const int nchunks = ((g.K + BK - 1) / BK + CH - 1) / CH;
      const float two_frac = __int_as_float((127 + a.frac) << 23);  // 2^frac
      int bz, m0, n0;
      decode_tile<BN>(g, t, bz, m0, n0);
      {
        const long long abz = a.A.batch == 1 ? 0 : bz, bbz = a.B.batch == 1 ? 0 : bz;
        if (et < BM) {
          const int i = m0 + et;
          const bool in = i < g.M;
          long long mr = -1;
          if (in && g.sym == SYM_ROWCOL) mr = g.c_c.at(i);
          long long ri = i;  // the pair's index for a packed-triangle row
          if (in && g.sym == SYM_TRIROW) {
            int mm, nn;
            tri_pair(i, g.pair_n, mm, nn);
            ri = (long long)mm * g.pair_n + nn;
            if (nn > mm) mr = g.c_r.at((long long)nn * g.pair_n + mm);
          }
          e_roff[et] = in ? g.c_r.at(ri) : 0;
          e_mr[et] = mr;
          e_srow[et] = in ? a.A.exps[abz * g.M + i] : 0;
        } else if (et < BM + BN) {
          const int c = et - BM, jj = n0 + c;
          const bool in = jj < g.N;
          long long mc = -1;
          if (in && g.sym == SYM_ROWCOL) mc = g.c_r.at(jj);
          long long cj = jj;
          if (in && g.sym == SYM_TRICOL) {
            int mm, nn;
            tri_pair(jj, g.pair_n, mm, nn);
            cj = (long long)mm * g.pair_n + nn;
            if (nn > mm) mc = g.c_c.at((long long)nn * g.pair_n + mm);
          }
          e_coff[c] = in ? g.c_c.at(cj) : 0;
          e_mc[c] = mc;
          e_scol[c] = in ? a.B.exps[bbz * g.N + jj] - 7 * gE - a.frac : 0;
        }
      }
      epi_barrier_any(false);  // tables visible
      const int n_valid = min(BN, g.N - n0);
      const bool cols_live = cg * CW < n_valid;  // warp-uniform
      long long R[CW];
#pragma unroll
      for (int j = 0; j < CW; ++j) R[j] = 0;
      bool ok = true;
      for (int c = 0; c < nchunks; ++c) {
        const bool got = mbar_wait(accfull_bar, (uint32_t)(gch & 1), abort_flag, a0.wait_ns);
        if (!__all_sync(0xffffffffu, got)) {
          signal_abort(abort_flag);
          ok = false;
          break;
        }
        tc_fence_after();
        const int fr = g.fdrain ? a.frac : 0;
        if (cols_live) drain_exact<BN, gE, CW>(lbase, R, fr);
        const bool last = c == nchunks - 1;
        if (has_inexact && cols_live && (g.fdrain || last)) {
          // the FP32 group: drained every chunk (fdrain) or folded in at the end
#pragma unroll
          for (int h = 0; h < CW / 8; ++h) {
            uint32_t v[8];
            tmem_ld8_async(lbase + (uint32_t)(3 * BN + h * 8), v);
            tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const long long f = split_round(__uint_as_float(v[j]) * upE, a.frac, two_frac);
              R[h * 8 + j] = g.fdrain ? R[h * 8 + j] + f : (long long)((unsigned long long)R[h * 8 + j] << a.frac) + f;
            }
          }
        } else if (last && !g.fdrain) {
#pragma unroll
          for (int j = 0; j < CW; ++j) R[j] = (long long)((unsigned long long)R[j] << a.frac);
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(accempty_bar);  // TMEM free for the next chunk / tile
        ++gch;
      }
      if (!ok) continue;  // the next tile's barrier sees the abort flag in every warp
      // convert and store from registers (rows are the output's unit stride)
      double* Cb = g.C + (long long)bz * g.c_sb;
      const bool mirror_rc = (g.sym == SYM_ROWCOL) && (m0 != n0);
      const int rlim = min(BM, g.M - m0), clim = min(BN, g.N - n0);
      if (row < rlim) {
        const int srow = e_srow[row];
        const long long ro = e_roff[row], mr = e_mr[row];
#pragma unroll
        for (int j = 0; j < CW; ++j) {
          const int c = cg * CW + j;
          if (c >= clim) continue;
          const double val = scaled_to_double(R[j], srow + e_scol[c], g.negate);
          const long long co = e_coff[c];
          Cb[ro + co] = val;
          if (mirror_rc) {
            Cb[e_mc[c] + mr] = val;
          } else if (g.sym == SYM_TRICOL) {
            const long long mc = e_mc[c];
            if (mc >= 0) Cb[ro + mc] = val;
          } else if (g.sym == SYM_TRIROW) {
            if (mr >= 0) Cb[mr + co] = val;
          }
        }
      }
    }
  }

  __syncthreads();
  // after an abort, the producer's copies land before the CTA exits
  if (warp == 0 && lane == 0 && *abort_flag) {
    for (int k = gkb_issued > STAGES ? gkb_issued - STAGES : 0; k < gkb_issued; ++k)
      mbar_wait(full_bar(k % STAGES), (uint32_t)((k / STAGES) & 1), nullptr, a0.wait_ns);
  }
  if (warp == 1) {
    if (*abort_flag) mbar_wait(done_bar, 0, nullptr, a0.wait_ns);
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(T::TMEM_COLS) : "memory");
  }
}

template <int S, int BN>
__global__ void __maxnreg__(MAX_REGS) ozaki_persistent_kernel(const __grid_constant__ KArgs a, int ntiles) {
  extern __shared__ unsigned char smem_raw[];
  if (*(volatile int*)&g_tc_status != 0) return;
  cta_persistent<S, BN, false>(a, nullptr, nullptr, 1, ntiles, a.g.tile_counter, smem_raw);
}

// Grouped persistent launch: problem p owns the tiles [starts[p], starts[p + 1])
// of one tile space walked in order through `counter` (caller memory, zeroed
// before the launch), one CTA per SM.
template <int S, int BN>
__global__ void __maxnreg__(MAX_REGS)
    ozaki_persistent_grouped_kernel(const KArgs* __restrict__ probs, const long long* __restrict__ starts, int nprob,
                                    int ntiles, unsigned int* counter) {
  extern __shared__ unsigned char smem_raw[];
  if (*(volatile int*)&g_tc_status != 0) return;
  cta_persistent<S, BN, true>(probs[0], probs, starts, nprob, ntiles, counter, smem_raw);
}

template <int S, int BN, int KIND>
__global__ void __maxnreg__(MAX_REGS) ozaki_kernel(const __grid_constant__ KArgs a) {
  extern __shared__ unsigned char smem_raw[];
  // a CTA of this or an earlier launch gave up: do not start (the host sees the status word)
  if (*(volatile int*)&g_tc_status != 0) return;
  int bz, m0, n0;
  if (!decode_tile<BN>(a.g, (long long)blockIdx.x + (long long)blockIdx.y * gridDim.x, bz, m0, n0)) return;
  cta_tile<S, BN, KIND>(a, bz, m0, n0, smem_raw);
}

// Grouped launch: problem p owns the tiles [starts[p], starts[p + 1]).
template <int S, int BN, int KIND>
__global__ void __maxnreg__(MAX_REGS)
    ozaki_grouped_kernel(const KArgs* __restrict__ probs, const long long* __restrict__ starts, int nprob) {
  extern __shared__ unsigned char smem_raw[];
  if (*(volatile int*)&g_tc_status != 0) return;
  const long long t = (long long)blockIdx.x + (long long)blockIdx.y * gridDim.x;
  int lo = 0, hi = nprob;  // find p with starts[p] <= t < starts[p + 1]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (starts[mid] <= t) lo = mid; else hi = mid;
  }
  if (t >= starts[nprob]) return;
  const KArgs& a = probs[lo];
  int bz, m0, n0;
  if (!decode_tile<BN>(a.g, t - starts[lo], bz, m0, n0)) return;
  cta_tile<S, BN, KIND>(a, bz, m0, n0, smem_raw);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// `code`: split code (1..6 digit slices or SPLIT_TF32X3)
size_t smem_bytes(int code, int BN) {
  const int S = form_of(code).S;
  const size_t stages = (size_t)STAGES * S * (TILE_BYTES + BN * SL_K * 2);
  const size_t zs = (size_t)BM * (BN + 1) * 8;
  return (stages > zs ? stages : zs) + epi_table_bytes(BN) + 256 + 1024;
}

using KernelFn = void (*)(KArgs);
using GroupedFn = void (*)(const KArgs*, const long long*, int);

template <int BN>
KernelFn single_for(int S) {
  switch (S) {
    case 1: return ozaki_kernel<1, BN, 0>;
    case 2: return ozaki_kernel<2, BN, 0>;
    case 3: return ozaki_kernel<3, BN, 0>;
    case 4: return ozaki_kernel<4, BN, 0>;
    case 5: return ozaki_kernel<5, BN, 0>;
    case SPLIT_TF32X3: return ozaki_kernel<2, BN, 1>;
    default: return ozaki_kernel<6, BN, 0>;
  }
}

template <int BN>
GroupedFn grouped_for(int S) {
  switch (S) {
    case 1: return ozaki_grouped_kernel<1, BN, 0>;
    case 2: return ozaki_grouped_kernel<2, BN, 0>;
    case 3: return ozaki_grouped_kernel<3, BN, 0>;
    case 4: return ozaki_grouped_kernel<4, BN, 0>;
    case 5: return ozaki_grouped_kernel<5, BN, 0>;
    case SPLIT_TF32X3: return ozaki_grouped_kernel<2, BN, 1>;
    default: return ozaki_grouped_kernel<6, BN, 0>;
  }
}

using PersistFn = void (*)(KArgs, int);
PersistFn persistent_for(int S) {
  switch (S) {
    case 1: return ozaki_persistent_kernel<1, 128>;
    case 2: return ozaki_persistent_kernel<2, 128>;
    case 3: return ozaki_persistent_kernel<3, 128>;
    case 4: return ozaki_persistent_kernel<4, 128>;
    case 5: return ozaki_persistent_kernel<5, 128>;
    default: return ozaki_persistent_kernel<6, 128>;
  }
}

using PersistGroupedFn = void (*)(const KArgs*, const long long*, int, int, unsigned int*);
PersistGroupedFn persistent_grouped_for(int S) {
  switch (S) {
    case 1: return ozaki_persistent_grouped_kernel<1, 128>;
    case 2: return ozaki_persistent_grouped_kernel<2, 128>;
    case 3: return ozaki_persistent_grouped_kernel<3, 128>;
    case 4: return ozaki_persistent_grouped_kernel<4, 128>;
    case 5: return ozaki_persistent_grouped_kernel<5, 128>;
    default: return ozaki_persistent_grouped_kernel<6, 128>;
  }
}

KernelFn kernel_for(int S, int BN) {
  return BN == 32 ? single_for<32>(S) : BN == 64 ? single_for<64>(S) : single_for<128>(S);
}
GroupedFn grouped_kernel_for(int S, int BN) {
  return BN == 32 ? grouped_for<32>(S) : BN == 64 ? grouped_for<64>(S) : grouped_for<128>(S);
}

// Opt every instantiation in to its dynamic shared memory once per device
// context (again after a cudaDeviceReset, whose new context has a new id).
int g_num_sms[64] = {0};

int configure_device() {
  static std::mutex mu;
  static unsigned long long configured[64] = {0};  // context id configured on each device
  int dev = 0;
  GB_TRY(cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lk(mu);
  if (dev < 0 || dev >= 64 || (ctx != 0 && configured[dev] == ctx)) return GB_OK;
  for (int bn : {32, 64, 128})
    for (int sl : {1, 2, 3, 4, 5, 6, SPLIT_TF32X3}) {
      const int sm = (int)smem_bytes(sl, bn);
      GB_TRY(cuda_status(cudaFuncSetAttribute(kernel_for(sl, bn), cudaFuncAttributeMaxDynamicSharedMemorySize, sm),
                         "cudaFuncSetAttribute"));
      GB_TRY(cuda_status(
          cudaFuncSetAttribute(grouped_kernel_for(sl, bn), cudaFuncAttributeMaxDynamicSharedMemorySize, sm),
          "cudaFuncSetAttribute"));
    }
  for (int sl = 1; sl <= 6; ++sl) {
    GB_TRY(cuda_status(cudaFuncSetAttribute(persistent_for(sl), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem_bytes(sl, 128)),
                       "cudaFuncSetAttribute"));
    GB_TRY(cuda_status(cudaFuncSetAttribute(persistent_grouped_for(sl), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem_bytes(sl, 128)),
                       "cudaFuncSetAttribute"));
  }
  GB_TRY(cuda_status(cudaDeviceGetAttribute(&g_num_sms[dev], cudaDevAttrMultiProcessorCount, dev),
                     "cudaDeviceGetAttribute"));
  configured[dev] = current_context_id();
  return GB_OK;
}

// Fraction bits of the fixed-point assembly: keep |z| < 2^62.
int frac_bits(int S, int K) {
  if (S == SPLIT_TF32X3) return 0;
  const int nkb = (K + BK - 1) / BK;
  const int nchunks = (nkb + CH - 1) / CH;
  const int gE = S + 1 < 4 ? S + 1 : 4;
  int lg = 0;
  while ((1 << lg) < nchunks) ++lg;
  const int rbits = lg + 22 + 7 * (gE - 2) + 2;
  int frac = 62 - rbits;
  if (frac > 16) frac = 16;
  if (frac < 0) frac = 0;
  return frac;
}

int check_problem(const SlicedDesc& A, const SlicedDesc& B, const OzGemm& g) {
  const SliceForm f = form_of(g.S);
  GB_REQUIRE(valid_split(g.S) && A.S == f.S && B.S == f.S && A.kind == f.kind && B.kind == f.kind,
             GB_ERR_INVALID_ARG, "ozaki_gemm: split form mismatch (code %d)", g.S);
  GB_REQUIRE(g.bn == 32 || g.bn == 64 || g.bn == 128, GB_ERR_INVALID_ARG, "ozaki_gemm: N tile %d not in {32,64,128}",
             g.bn);
  GB_REQUIRE(A.rows == g.M && B.rows == g.N && A.K == g.K && B.K == g.K && (A.batch == g.batch || A.batch == 1) &&
                 (B.batch == g.batch || B.batch == 1),
             GB_ERR_BAD_SHAPE, "ozaki_gemm: operand shapes do not match the GEMM");
  GB_REQUIRE(g.sym != SYM_ROWCOL || (g.M == g.N && g.bn == BM), GB_ERR_BAD_SHAPE,
             "ozaki_gemm: SYM_ROWCOL needs M == N and 128-wide tiles");
  GB_REQUIRE(g.sym != SYM_PAIRCOL, GB_ERR_INVALID_ARG,
             "ozaki_gemm: pair symmetry runs over the packed pair triangle here (SYM_TRIROW / SYM_TRICOL)");
  GB_REQUIRE(g.sym != SYM_TRIROW || (long long)g.pair_n * (g.pair_n + 1) / 2 == g.M, GB_ERR_BAD_SHAPE,
             "ozaki_gemm: SYM_TRIROW needs M == pair_n (pair_n + 1) / 2");
  GB_REQUIRE(g.sym != SYM_TRICOL || (long long)g.pair_n * (g.pair_n + 1) / 2 == g.N, GB_ERR_BAD_SHAPE,
             "ozaki_gemm: SYM_TRICOL needs N == pair_n (pair_n + 1) / 2");
  GB_REQUIRE(g.K > 0 && g.batch <= 65535, GB_ERR_BAD_SHAPE, "ozaki_gemm: bad K or batch");
  GB_REQUIRE((reinterpret_cast<uintptr_t>(A.planes) & 15) == 0 && (reinterpret_cast<uintptr_t>(B.planes) & 15) == 0,
             GB_ERR_INVALID_ARG, "ozaki_gemm: slice planes not 16-byte aligned");
  return GB_OK;
}

constexpr unsigned long long kDefaultWaitNs = 2000000000ull;  // 2 s per wait
std::atomic<unsigned long long> g_wait_limit_ns{kDefaultWaitNs};
std::atomic<int> g_withhold_stage{-1};

KArgs make_args(const SlicedDesc& A, const SlicedDesc& B, const OzGemm& g) {
  KArgs ka{g, A, B, frac_bits(g.S, g.K), g_wait_limit_ns.load(), g_withhold_stage.load()};
  if (g.K > 4096 && g.S != SPLIT_TF32X3) ka.g.fdrain = 1;
  return ka;
}

dim3 grid_for(long long tiles) {
  // x up to 2^31 - 1; split very large tile counts over y
  const long long gx = tiles < 2147483647LL ? tiles : 65536;
  return dim3((unsigned)gx, (unsigned)((tiles + gx - 1) / gx));
}

int launch_error(const char* tag, cudaError_t le, int S, int BN) {
  char info[512];
  ozaki_kernel_info(info, sizeof(info));
  set_error(GB_ERR_CUDA, "%s: %s (S=%d BN=%d threads %d, dynamic smem %zu; %s)", tag, cudaGetErrorString(le), S, BN,
            THREADS, smem_bytes(S, BN), info);
  return GB_ERR_CUDA;
}

}  // namespace

long long ozaki_tiles(const OzGemm& g) {
  return ((long long)(g.M + BM - 1) / BM) * ((g.N + g.bn - 1) / g.bn) * (long long)g.batch;
}

int ozaki_gemm(const SlicedDesc& A, const SlicedDesc& B, const OzGemm& g, cudaStream_t stream) {
  if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return GB_OK;
  GB_TRY(check_problem(A, B, g));
  GB_TRY(configure_device());
  const KArgs ka = make_args(A, B, g);
  const long long tiles = ozaki_tiles(g);
  // outputs whose tile rows are the unit stride take the persistent kernel
  const bool rows_fast = !(g.c_c.div == 0 && g.c_c.s0 == 1) && (g.c_r.div == 0 && g.c_r.s0 == 1);
  int dev = 0;
  cudaGetDevice(&dev);
  const int nsm = (dev >= 0 && dev < 64 && g_num_sms[dev] > 0) ? g_num_sms[dev] : 0;
  if (g.S >= 1 && g.S <= 6 && g.bn == 128 && rows_fast && nsm > 0 && tiles < (1LL << 30)) {
    const long long grid = tiles < nsm ? tiles : nsm;
    KArgs kp = ka;
    if (g.tile_counter && tiles > grid) {
      GB_TRY(cuda_status(cudaMemsetAsync(g.tile_counter, 0, sizeof(unsigned int), stream), "tile counter"));
    } else {
      kp.g.tile_counter = nullptr;  // one tile per CTA, or the static walk
    }
    const int pi = prof_begin(g.tag, stream);
    persistent_for(g.S)<<<(unsigned)grid, THREADS, smem_bytes(g.S, 128), stream>>>(kp, (int)tiles);
    prof_end(pi, stream);
  } else {
    const int pi = prof_begin(g.tag, stream);
    kernel_for(g.S, g.bn)<<<grid_for(tiles), THREADS, smem_bytes(g.S, g.bn), stream>>>(ka);
    prof_end(pi, stream);
  }
  const cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) return launch_error(g.tag, le, g.S, g.bn);
  return GB_OK;
}

// table layout: KArgs[nprob] | starts[nprob + 1] | tile counter
size_t ozaki_group_table_bytes(int nprob) {
  return align256((size_t)nprob * sizeof(KArgs)) + align256((size_t)(nprob + 1) * sizeof(long long)) + 256;
}

int ozaki_group_upload(const OzProblem* probs, int nprob, void* table, bool* persistent) {
  GB_REQUIRE(nprob >= 1 && probs && table, GB_ERR_INVALID_ARG, "ozaki_group_upload: empty group");
  std::vector<KArgs> args;
  std::vector<long long> starts(1, 0);
  bool all_rows_fast = true;
  for (int i = 0; i < nprob; ++i) {
    GB_TRY(check_problem(probs[i].A, probs[i].B, probs[i].g));
    GB_REQUIRE(probs[i].g.S == probs[0].g.S && probs[i].g.bn == probs[0].g.bn, GB_ERR_INVALID_ARG,
               "ozaki_group_upload: a group shares one slice count and tile width");
    args.push_back(make_args(probs[i].A, probs[i].B, probs[i].g));
    starts.push_back(starts.back() + ozaki_tiles(probs[i].g));
    const OzGemm& g = probs[i].g;
    all_rows_fast = all_rows_fast && !(g.c_c.div == 0 && g.c_c.s0 == 1) && (g.c_r.div == 0 && g.c_r.s0 == 1);
  }
  // the persistent form stores from the epilogue's registers: every output's
  // tile rows must be its unit stride; bf16 digits and 128-wide tiles
  if (persistent)
    *persistent = all_rows_fast && probs[0].g.S >= 1 && probs[0].g.S <= 6 && probs[0].g.bn == 128 &&
                  starts.back() < (1LL << 30);
  char* t = static_cast<char*>(table);
  GB_TRY(cuda_status(cudaMemcpy(t, args.data(), nprob * sizeof(KArgs), cudaMemcpyHostToDevice), "group table"));
  GB_TRY(cuda_status(cudaMemcpy(t + align256((size_t)nprob * sizeof(KArgs)), starts.data(),
                                (nprob + 1) * sizeof(long long), cudaMemcpyHostToDevice),
                     "group table"));
  return GB_OK;
}

int ozaki_gemm_grouped(const void* table, int nprob, long long total_tiles, int S, int bn, cudaStream_t stream,
                       const char* tag, bool persistent) {
  if (total_tiles <= 0) return GB_OK;
  GB_TRY(configure_device());
  const char* t = static_cast<const char*>(table);
  const KArgs* probs = reinterpret_cast<const KArgs*>(t);
  const size_t off_starts = align256((size_t)nprob * sizeof(KArgs));
  const long long* starts = reinterpret_cast<const long long*>(t + off_starts);
  int dev = 0;
  cudaGetDevice(&dev);
  const int nsm = (dev >= 0 && dev < 64 && g_num_sms[dev] > 0) ? g_num_sms[dev] : 0;
  if (persistent && S >= 1 && S <= 6 && bn == 128 && nsm > 0 && total_tiles < (1LL << 30)) {
    // one CTA per SM walking the concatenated tile space in order
    unsigned int* counter = reinterpret_cast<unsigned int*>(
        const_cast<char*>(t) + off_starts + align256((size_t)(nprob + 1) * sizeof(long long)));
    const long long grid = total_tiles < nsm ? total_tiles : nsm;
    GB_TRY(cuda_status(cudaMemsetAsync(counter, 0, sizeof(unsigned int), stream), "grouped tile counter"));
    const int pi = prof_begin(tag, stream);
    persistent_grouped_for(S)<<<(unsigned)grid, THREADS, smem_bytes(S, 128), stream>>>(probs, starts, nprob,
                                                                                      (int)total_tiles, counter);
    prof_end(pi, stream);
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return launch_error(tag, le, S, 128);
    return GB_OK;
  }
  const int pi = prof_begin(tag, stream);
  grouped_kernel_for(S, bn)<<<grid_for(total_tiles), THREADS, smem_bytes(S, bn), stream>>>(probs, starts, nprob);
  prof_end(pi, stream);
  const cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) return launch_error(tag, le, S, bn);
  return GB_OK;
}

int ozaki_status(int reset, int* out) {
  int v = 0;
  GB_TRY(cuda_status(cudaMemcpyFromSymbol(&v, g_tc_status, sizeof(int)), "read tensor-core status"));
  if (reset) {
    const int zero = 0;
    GB_TRY(cuda_status(cudaMemcpyToSymbol(g_tc_status, &zero, sizeof(int)), "reset tensor-core status"));
  }
  *out = v;
  return GB_OK;
}

int* device_status_word() {
  static std::mutex mu;
  static unsigned long long ctx_ids[64] = {0};
  static int* addrs[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  const unsigned long long id = current_context_id();
  std::lock_guard<std::mutex> lk(mu);
  if (addrs[dev] == nullptr || id == 0 || ctx_ids[dev] != id) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_tc_status) != cudaSuccess) return nullptr;
    addrs[dev] = static_cast<int*>(p);
    ctx_ids[dev] = current_context_id();
  }
  return addrs[dev];
}

// The two driver functions come through the runtime's entry-point query, so
// the library keeps no link-time dependency on the driver library (it loads
// on a machine without a GPU, where only its size queries are used).
unsigned long long current_context_id() {
  using GetCurrentFn = CUresult (*)(CUcontext*);
  using GetIdFn = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetIdFn>(f);
  });
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return 0;
  unsigned long long id = 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

int ozaki_kernel_info(char* out, size_t len) {
  cudaFuncAttributes fa{};
  cudaError_t e = cudaFuncGetAttributes(&fa, kernel_for(6, 128));
  int occ = -1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel_for(6, 128), THREADS, smem_bytes(6, 128));
  int dev = 0, regs_sm = 0, smem_optin = 0, max_thr = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaDeviceGetAttribute(&max_thr, cudaDevAttrMaxThreadsPerBlock, dev);
  snprintf(out, len,
           "attr=%s regs=%d maxThreadsPerBlock=%d localBytes=%zu staticSmem=%zu maxDynSmem=%d occupancy=%d "
           "regsPerSM=%d smemOptin=%d devMaxThreads=%d",
           cudaGetErrorString(e), fa.numRegs, fa.maxThreadsPerBlock, fa.localSizeBytes, fa.sharedSizeBytes,
           fa.maxDynamicSharedSizeBytes, occ, regs_sm, smem_optin, max_thr);
  return GB_OK;
}

}  // namespace gb

extern "C" int gb_set_wait_limit_ns(unsigned long long limit_ns) {
  gb::clear_error();
  gb::g_wait_limit_ns.store(limit_ns ? limit_ns : gb::kDefaultWaitNs);
  return GB_OK;
}

extern "C" int gb_test_withhold_stage(int stage) {
  gb::clear_error();
  gb::g_withhold_stage.store(stage < 0 ? -1 : stage);
  return GB_OK;
}
