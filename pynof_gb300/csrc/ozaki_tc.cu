// tcgen05 split-product FP64 GEMM (see ozaki_tc.cuh).
//
// CTA: 18 warps.  warp 0 lane 0 is the producer: a 4-stage ring in which every
// stage holds the S slices of a 128 x 16 block of A and of B, each operand one
// contiguous cp.async.bulk copy (the slicer stores the digits in the
// tensor-core core-matrix order, slice.cuh).  warp 1 allocates TMEM (512
// columns) and its lane 0 issues tcgen05.mma (M=128, N=128, K=16,
// bf16 -> f32).  warps 2..17 drain and finish: warp w reads TMEM lanes
// 32 (w % 4) .. +31 (tile rows) and columns 32 ((w - 2) / 4) .. +31 of every
// accumulator.
//
// TMEM columns: [0,128) group 2, [128,256) group 3, [256,384) group 4 (exact,
// drained every 12 stages = 192 k), [384,512) groups 5.. (whole K).
//
// Every mbarrier wait is bounded (kWaitLimitNs); on timeout the CTA records
// GB_ERR_TIMEOUT in the device status word, stops issuing work, waits (bounded)
// for its own TMA copies and MMAs in flight, frees TMEM and exits.
#include <cuda_bf16.h>

#include <cstdio>
#include <mutex>

#include "ozaki_tc.cuh"

static __device__ int g_tc_status;

namespace gb {
namespace {

constexpr int BM = 128, BN = 128, BK = SL_K, STAGES = 4, CH = 12;
constexpr int NUM_EPI_WARPS = 16, THREADS = 32 * (2 + NUM_EPI_WARPS);
// 18 warps put 5 warps on two of the four SM sub-partitions, whose register
// files hold 16K registers each: 5 * 32 * 96 <= 16384 caps the kernel at 96.
constexpr int MAX_REGS = 96;
constexpr uint32_t TILE_BYTES = SL_TILE_BYTES;  // 4 KB per slice tile (BM == BN == SL_ROWS)
constexpr uint32_t TMEM_COLS = 512;
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s per wait
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

// Bounded wait.  Returns false on timeout, or (if abort_flag != nullptr) as soon
// as another role has aborted.
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = now_ns();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try(bar, parity)) return true;
    if (abort_flag && *abort_flag) return false;
    if ((it & 63) == 0 && now_ns() - t0 > kWaitLimitNs) return false;
  }
}

__device__ __forceinline__ void signal_abort(volatile int* abort_flag) {
  *abort_flag = 1;
  atomicExch(&g_tc_status, GB_ERR_TIMEOUT);
}

// Contiguous global -> shared bulk copy completing on an mbarrier.
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// UMMA shared-memory descriptor of one 128 x 16 slice tile: K-major, no
// swizzle; core matrices (8 rows x 16 B) 2 KB apart along K (leading byte
// offset) and 128 B apart along the rows (stride byte offset).
__device__ __forceinline__ uint64_t desc_tile(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)(2048u >> 4) << 16;   // leading byte offset
  d |= (uint64_t)(128u >> 4) << 32;    // stride byte offset
  d |= (uint64_t)1 << 46;              // descriptor version
  return d;                            // layout type 0: no swizzle
}

// kind::f16 instruction descriptor: bf16 x bf16 -> f32, both K-major, M=128, N=128.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, bool accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(IDESC), "r"((uint32_t)accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&v)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// int64 fixed point z * 2^scale -> double, round to nearest even, integer ops only.
__device__ __forceinline__ double fixed_to_double(long long z, int scale, int negate) {
  if (z == 0) return 0.0;
  unsigned long long sign = 0;
  unsigned long long u = (unsigned long long)z;
  if (z < 0) {
    sign = 1ull << 63;
    u = 0ull - u;
  }
  sign ^= (unsigned long long)(negate != 0) << 63;
  int top = 63 - __clzll((long long)u);  // index of the leading one
  unsigned long long mant;
  if (top > 52) {
    const int sh = top - 52;
    mant = u >> sh;
    const unsigned long long rem = u & ((1ull << sh) - 1);
    const unsigned long long half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (mant & 1ull))) {
      ++mant;
      if (mant == (1ull << 53)) {
        mant >>= 1;
        ++top;
      }
    }
  } else {
    mant = u << (52 - top);
  }
  const long long ef = (long long)top + scale + 1023;
  if (ef <= 0) return __longlong_as_double((long long)sign);                           // underflow -> 0
  if (ef >= 2047) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));  // overflow -> inf
  return __longlong_as_double((long long)(sign | ((unsigned long long)ef << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

struct KArgs {
  OzGemm g;
  SlicedDesc A, B;
  int frac;
};

// MMAs of one stage, fully unrolled for S slices: a product (s, t) reads slice
// tile s of A and t of B, whose descriptors differ from the stage's first tile
// descriptors only in the start-address field (+ (s - 1) * TILE_BYTES / 16).
template <int S>
__device__ __forceinline__ void issue_inexact(uint32_t tmem, uint64_t da, uint64_t db, bool& started) {
#pragma unroll
  for (int s = 1; s <= S; ++s)
#pragma unroll
    for (int t = 1; t <= S + 1 - s; ++t) {
      if (s + t <= 4) continue;
      mma_bf16(tmem + 384, da + (uint64_t)((s - 1) * (TILE_BYTES >> 4)), db + (uint64_t)((t - 1) * (TILE_BYTES >> 4)),
               started);
      started = true;
    }
}

template <int S>
__device__ __forceinline__ void issue_exact(uint32_t tmem, uint64_t da, uint64_t db, bool first) {
  constexpr int gE = (S + 1) < 4 ? (S + 1) : 4;
#pragma unroll
  for (int gg = 2; gg <= gE; ++gg) {
#pragma unroll
    for (int s = 1; s < gg; ++s) {
      const int t = gg - s;
      if (s > S || t > S) continue;
      mma_bf16(tmem + (gg - 2) * 128, da + (uint64_t)((s - 1) * (TILE_BYTES >> 4)),
               db + (uint64_t)((t - 1) * (TILE_BYTES >> 4)), !(first && s == 1));
    }
  }
}

template <int SLICES>
__global__ void __maxnreg__(MAX_REGS) ozaki_kernel(const __grid_constant__ KArgs a) {
  extern __shared__ unsigned char smem_raw[];
  const OzGemm& g = a.g;
  // M tiles vary fastest, so the CTAs that share a B tile run together and the
  // B slices are read from HBM once (L2 serves the other M tiles).
  const int mtiles = (g.M + BM - 1) / BM;
  const int m0 = (int)(blockIdx.x % mtiles) * BM;
  const int n0 = (int)(blockIdx.x / mtiles) * BN;
  const int bz = blockIdx.y;

  if (g.sym == SYM_ROWCOL && m0 > n0) return;
  if (g.sym == SYM_PAIRCOL) {
    const int j1 = min(n0 + BN, g.N) - 1;
    const int ma = n0 / g.pair_n, mb = j1 / g.pair_n;
    if (ma == mb && (j1 % g.pair_n) < ma) return;
  }
  // a CTA of this or an earlier launch gave up: do not start (the host sees the status word)
  if (*(volatile int*)&g_tc_status != 0) return;

  constexpr int S = SLICES;
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const uint32_t stage_bytes = 2u * S * TILE_BYTES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * stage_bytes);
  // bars: full[STAGES], empty[STAGES], accfull, accempty, done
  volatile uint32_t* tmem_slot = reinterpret_cast<volatile uint32_t*>(bars + 2 * STAGES + 4);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 2 * STAGES + 5);
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
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(const_cast<uint32_t*>(tmem_slot))),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    tc_fence_before();
  }
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  const int nkb = (g.K + BK - 1) / BK;
  const int nchunks = (nkb + CH - 1) / CH;
  const int gE = min(S + 1, 4);
  const bool has_inexact = (S + 1) > 4;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int issued = 0;
      const uint32_t half = (uint32_t)S * TILE_BYTES;
      // an operand sliced once (batch 1) is shared by every batch entry
      const long long abz = a.A.batch == 1 ? 0 : bz, bbz = a.B.batch == 1 ? 0 : bz;
      const unsigned char* ga = reinterpret_cast<const unsigned char*>(a.A.planes) + abz * a.A.batch_bytes() +
                                (long long)(m0 / BM) * a.A.kblocks() * half;
      const unsigned char* gb_ = reinterpret_cast<const unsigned char*>(a.B.planes) + bbz * a.B.batch_bytes() +
                                 (long long)(n0 / BN) * a.B.kblocks() * half;
      for (int kb = 0; kb < nkb; ++kb) {
        const int st = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!mbar_wait(empty_bar(st), ph ^ 1, abort_flag)) {
          signal_abort(abort_flag);
          break;
        }
        mbar_expect_tx(full_bar(st), stage_bytes);
        const uint32_t sa = sbase + st * stage_bytes;
        bulk_load(sa, ga + (long long)kb * half, half, full_bar(st));
        bulk_load(sa + half, gb_ + (long long)kb * half, half, full_bar(st));
        ++issued;
      }
      if (*abort_flag) {
        // let the copies this thread issued land before the CTA exits
        for (int kb = max(0, issued - STAGES); kb < issued; ++kb)
          mbar_wait(full_bar(kb % STAGES), (kb / STAGES) & 1, nullptr);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      bool f_started = false;
      for (int kb = 0; kb < nkb; ++kb) {
        const int st = kb % STAGES;
        if (!mbar_wait(full_bar(st), (kb / STAGES) & 1, abort_flag)) {
          signal_abort(abort_flag);
          break;
        }
        tc_fence_after();
        const uint32_t sa = sbase + st * stage_bytes;
        const uint64_t da = desc_tile(sa), db = desc_tile(sa + S * TILE_BYTES);
        const int c = kb / CH;
        const bool first = (kb % CH) == 0;
        if (g.fdrain) {
          // the FP32 accumulator is drained with the exact groups: restart it every chunk
          if (first && c > 0) {
            if (!mbar_wait(accempty_bar, (c - 1) & 1, abort_flag)) {
              signal_abort(abort_flag);
              break;
            }
            tc_fence_after();
          }
          if (first) f_started = false;
          if (has_inexact) issue_inexact<S>(tmem, da, db, f_started);
        } else {
          if (has_inexact) issue_inexact<S>(tmem, da, db, f_started);
          if (first && c > 0) {
            if (!mbar_wait(accempty_bar, (c - 1) & 1, abort_flag)) {
              signal_abort(abort_flag);
              break;
            }
            tc_fence_after();
          }
        }
        issue_exact<S>(tmem, da, db, first);
        if ((kb % CH) == CH - 1 || kb == nkb - 1) mma_commit(accfull_bar);
        mma_commit(empty_bar(st));
      }
      mma_commit(done_bar);
    }
  } else {
    // ---------------- epilogue: drain exact groups, assemble FP64 ----------------
    const int q = warp & 3;
    const int cg = (warp - 2) >> 2;
    const uint32_t lbase = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(cg * 32);
    long long R[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) R[j] = 0;
    bool ok = true;
    for (int c = 0; c < nchunks; ++c) {
      const bool got = mbar_wait(accfull_bar, c & 1, abort_flag);
      if (!__all_sync(0xffffffffu, got)) {
        signal_abort(abort_flag);
        ok = false;
        break;
      }
      tc_fence_after();
      const int fr = g.fdrain ? a.frac : 0;  // fraction bits carried by R from the start
      for (int gg = 2; gg <= gE; ++gg) {
        const float up = __int_as_float((127 + 7 * gg) << 23);  // 2^(7 g)
        const int sh = 7 * (gE - gg) + fr;
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          uint32_t v[8];
          tmem_ld8(lbase + (uint32_t)((gg - 2) * 128 + h * 8), v);
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const float f = fmaf(__uint_as_float(v[j]), up, MAGIC);
            const long long iv = (long long)(__float_as_int(f) - MAGIC_BITS);
            R[h * 8 + j] += (long long)((unsigned long long)iv << sh);
          }
        }
      }
      if (has_inexact && g.fdrain) {
        const float upEF = __int_as_float((127 + 7 * gE + a.frac) << 23);  // 2^(7 gE + frac)
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          uint32_t v[8];
          tmem_ld8(lbase + 384u + (uint32_t)(h * 8), v);
#pragma unroll
          for (int j = 0; j < 8; ++j) R[h * 8 + j] += __float2ll_rn(__uint_as_float(v[j]) * upEF);
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(accempty_bar);
    }
    if (ok) {
      const bool got = mbar_wait(done_bar, 0, abort_flag);
      if (!__all_sync(0xffffffffu, got)) {
        signal_abort(abort_flag);
        ok = false;
      }
    }
    if (ok) {
      tc_fence_after();
      const int i = m0 + q * 32 + lane;
      const float upE = __int_as_float((127 + 7 * gE) << 23);
      const float upF = __int_as_float((127 + a.frac) << 23);
      const int ea = (i < g.M) ? a.A.exps[(a.A.batch == 1 ? 0LL : (long long)bz) * g.M + i] : 0;
      double* Cb = g.C + (long long)bz * g.c_sb;
      const long long ri = (i < g.M) ? g.c_r.at(i) : 0;
      const bool mirror_rc = (g.sym == SYM_ROWCOL) && (m0 != n0);
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        uint32_t v[8];
        if (has_inexact && !g.fdrain) {
          tmem_ld8(lbase + 384u + (uint32_t)(h * 8), v);
        } else {
#pragma unroll
          for (int j = 0; j < 8; ++j) v[j] = 0u;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int jj = n0 + cg * 32 + h * 8 + j;
          if (i >= g.M || jj >= g.N) continue;
          const float t = __uint_as_float(v[j]) * upE;
          const float th = rintf(t);
          const long long hi = __float2ll_rn(th);
          const long long lo = __float2ll_rn((t - th) * upF);
          const long long z = g.fdrain ? R[h * 8 + j]
                                       : (long long)((unsigned long long)(R[h * 8 + j] + hi) << a.frac) + lo;
          const int eb = a.B.exps[(a.B.batch == 1 ? 0LL : (long long)bz) * g.N + jj];
          const double val = fixed_to_double(z, ea + eb - 7 * gE - a.frac, g.negate);
          Cb[ri + g.c_c.at(jj)] = val;
          if (mirror_rc) {
            Cb[g.c_r.at(jj) + g.c_c.at(i)] = val;
          } else if (g.sym == SYM_PAIRCOL) {
            const int mm = jj / g.pair_n, nn = jj % g.pair_n;
            if (nn > mm) Cb[ri + g.c_c.at((long long)nn * g.pair_n + mm)] = val;
          }
        }
      }
    }
  }

  __syncthreads();
  if (warp == 1) {
    if (*abort_flag) {
      // every MMA this CTA issued must be complete before TMEM is released
      mbar_wait(done_bar, 0, nullptr);
    }
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
size_t smem_bytes(int S) { return (size_t)STAGES * 2 * S * TILE_BYTES + 256 + 1024; }

using KernelFn = void (*)(KArgs);
KernelFn kernel_for(int S) {
  switch (S) {
    case 1: return ozaki_kernel<1>;
    case 2: return ozaki_kernel<2>;
    case 3: return ozaki_kernel<3>;
    case 4: return ozaki_kernel<4>;
    case 5: return ozaki_kernel<5>;
    default: return ozaki_kernel<6>;
  }
}

}  // namespace

int ozaki_gemm(const SlicedDesc& A, const SlicedDesc& B, const OzGemm& g, cudaStream_t stream) {
  if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return GB_OK;
  GB_REQUIRE(g.S >= 1 && g.S <= 6 && A.S == g.S && B.S == g.S, GB_ERR_INVALID_ARG, "ozaki_gemm: nslices mismatch");
  GB_REQUIRE(A.rows == g.M && B.rows == g.N && A.K == g.K && B.K == g.K && (A.batch == g.batch || A.batch == 1) &&
                 (B.batch == g.batch || B.batch == 1),
             GB_ERR_BAD_SHAPE, "ozaki_gemm: operand shapes do not match the GEMM");
  GB_REQUIRE(g.sym != SYM_ROWCOL || g.M == g.N, GB_ERR_BAD_SHAPE, "ozaki_gemm: SYM_ROWCOL needs M == N");
  GB_REQUIRE(g.sym != SYM_PAIRCOL || (long long)g.pair_n * g.pair_n == g.N, GB_ERR_BAD_SHAPE,
             "ozaki_gemm: SYM_PAIRCOL needs N == pair_n^2");
  const long long tiles = ((g.M + BM - 1) / BM) * ((g.N + BN - 1) / BN);
  GB_REQUIRE(g.batch <= 65535 && tiles <= 2147483647LL, GB_ERR_BAD_SHAPE, "ozaki_gemm: grid too large");
  if (g.K == 0) {
    GB_REQUIRE(false, GB_ERR_BAD_SHAPE, "ozaki_gemm: K == 0");
  }
  GB_REQUIRE((reinterpret_cast<uintptr_t>(A.planes) & 15) == 0 && (reinterpret_cast<uintptr_t>(B.planes) & 15) == 0,
             GB_ERR_INVALID_ARG, "ozaki_gemm: slice planes not 16-byte aligned");
  const size_t smem = smem_bytes(g.S);
  static std::mutex mu;
  static int configured_dev[64] = {0};
  {
    int dev = 0;
    GB_TRY(cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 64 && !configured_dev[dev]) {
      for (int sl = 1; sl <= 6; ++sl)
        GB_TRY(cuda_status(cudaFuncSetAttribute(kernel_for(sl), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)smem_bytes(sl)),
                           "cudaFuncSetAttribute"));
      configured_dev[dev] = 1;
    }
  }
  // fraction bits of the fixed-point assembly: keep |z| < 2^62
  const int nkb = (g.K + BK - 1) / BK;
  const int nchunks = (nkb + CH - 1) / CH;
  const int gE = g.S + 1 < 4 ? g.S + 1 : 4;
  int lg = 0;
  while ((1 << lg) < nchunks) ++lg;
  const int rbits = lg + 22 + 7 * (gE - 2) + 2;
  int frac = 62 - rbits;
  if (frac > 16) frac = 16;
  if (frac < 0) frac = 0;
  KArgs ka{g, A, B, frac};
  if (g.K > 4096) ka.g.fdrain = 1;
  dim3 grid((unsigned)tiles, (unsigned)g.batch);
  const int pi = prof_begin(g.tag, stream);
  kernel_for(g.S)<<<grid, THREADS, smem, stream>>>(ka);
  prof_end(pi, stream);
  const cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) {
    char info[512];
    ozaki_kernel_info(info, sizeof(info));
    set_error(GB_ERR_CUDA, "%s: %s (threads %d, dynamic smem %zu; %s)", g.tag, cudaGetErrorString(le), THREADS,
              smem, info);
    return GB_ERR_CUDA;
  }
  return GB_OK;
}

int ozaki_kernel_info(char* out, size_t len) {
  cudaFuncAttributes fa{};
  cudaError_t e = cudaFuncGetAttributes(&fa, kernel_for(6));
  int occ = -1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel_for(6), THREADS, smem_bytes(6));
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

}  // namespace gb
