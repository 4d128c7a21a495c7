// tcgen05 split-product FP64 GEMM (see ozaki_tc.cuh).
//
// CTA: 18 warps.  warp 0 lane 0 issues TMA loads (2-stage ring, every stage
// holds the S slices of a 128 x 32 A tile and of a 128 x 32 B tile, 64-byte
// swizzled, K-major); warp 1 allocates TMEM (512 columns) and its lane 0
// issues tcgen05.mma (M=128, N=128, K=16, bf16 -> f32); warps 2..17 drain and
// finish: warp w reads TMEM lanes 32 (w % 4) .. +31 (tile rows) and columns
// 32 ((w - 2) / 4) .. +31 of every accumulator.
//
// TMEM columns: [0,128) group 2, [128,256) group 3, [256,384) group 4 (exact,
// drained every 6 stages = 192 k), [384,512) groups 5.. (whole K).
//
// Every mbarrier wait is bounded (kWaitLimitNs); on timeout the CTA records
// GB_ERR_TIMEOUT in the device status word, stops issuing work, waits (bounded)
// for its own TMA copies and MMAs in flight, frees TMEM and exits.
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdio>
#include <mutex>

#include "ozaki_tc.cuh"

static __device__ int g_tc_status;

namespace gb {
namespace {

constexpr int BM = 128, BN = 128, BK = 32, STAGES = 2, CH = 6;
constexpr int NUM_EPI_WARPS = 16, THREADS = 32 * (2 + NUM_EPI_WARPS);
// 18 warps put 5 warps on two of the four SM sub-partitions, whose register
// files hold 16K registers each: 5 * 32 * 96 <= 16384 caps the kernel at 96.
constexpr int MAX_REGS = 96;
constexpr uint32_t TILE_BYTES = BM * BK * 2;  // 8 KB per slice tile (BM == BN)
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

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
      : "memory");
}

// UMMA shared-memory descriptor: K-major, 64-byte swizzle, 8-row groups 512 B apart.
__device__ __forceinline__ uint64_t desc_sw64(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;              // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512u >> 4) << 32;    // stride byte offset
  d |= (uint64_t)1 << 46;              // descriptor version
  d |= (uint64_t)4 << 61;              // SWIZZLE_64B
  return d;
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

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
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
  const int* expA;
  const int* expB;
  int frac;
};

__global__ void __maxnreg__(MAX_REGS)
    ozaki_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const KArgs a) {
  extern __shared__ unsigned char smem_raw[];
  const OzGemm& g = a.g;
  const int m0 = blockIdx.y * BM;
  const int n0 = blockIdx.x * BN;
  const int bz = blockIdx.z;

  if (g.sym == SYM_ROWCOL && m0 > n0) return;
  if (g.sym == SYM_PAIRCOL) {
    const int j1 = min(n0 + BN, g.N) - 1;
    const int ma = n0 / g.pair_n, mb = j1 / g.pair_n;
    if (ma == mb && (j1 % g.pair_n) < ma) return;
  }
  // a CTA of this or an earlier launch gave up: do not start (the host sees the status word)
  if (*(volatile int*)&g_tc_status != 0) return;

  const int S = g.S;
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const uint32_t stage_bytes = 2u * S * TILE_BYTES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * stage_bytes);
  // bars: full[0..1], empty[0..1], accfull, accempty, done
  volatile uint32_t* tmem_slot = reinterpret_cast<volatile uint32_t*>(bars + 8);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 9);
  const uint32_t sbase = smem_u32(smem);
  const uint32_t bar0 = smem_u32(bars);
  auto full_bar = [&](int st) { return bar0 + 8u * st; };
  auto empty_bar = [&](int st) { return bar0 + 8u * (2 + st); };
  const uint32_t accfull_bar = bar0 + 8u * 4, accempty_bar = bar0 + 8u * 5, done_bar = bar0 + 8u * 6;

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
  if (warp == 0 && lane == 0) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
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
      for (int kb = 0; kb < nkb; ++kb) {
        const int st = kb & 1;
        const uint32_t ph = (kb >> 1) & 1;
        if (!mbar_wait(empty_bar(st), ph ^ 1, abort_flag)) {
          signal_abort(abort_flag);
          break;
        }
        mbar_expect_tx(full_bar(st), stage_bytes);
        const uint32_t sa = sbase + st * stage_bytes;
        for (int s = 0; s < S; ++s) tma_load_3d(sa + s * TILE_BYTES, &tmA, kb * BK, m0, bz * S + s, full_bar(st));
        for (int s = 0; s < S; ++s)
          tma_load_3d(sa + (S + s) * TILE_BYTES, &tmB, kb * BK, n0, bz * S + s, full_bar(st));
        ++issued;
      }
      if (*abort_flag) {
        // let the copies this thread issued land before the CTA exits
        for (int kb = max(0, issued - STAGES); kb < issued; ++kb) mbar_wait(full_bar(kb & 1), (kb >> 1) & 1, nullptr);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      bool f_started = false;
      for (int kb = 0; kb < nkb; ++kb) {
        const int st = kb & 1;
        if (!mbar_wait(full_bar(st), (kb >> 1) & 1, abort_flag)) {
          signal_abort(abort_flag);
          break;
        }
        tc_fence_after();
        const uint32_t sa = sbase + st * stage_bytes;
        const uint32_t sb = sa + S * TILE_BYTES;
        if (has_inexact) {
          for (int s = 1; s <= S; ++s)
            for (int t = 1; t <= S + 1 - s; ++t) {
              if (s + t <= 4) continue;
              for (int ks = 0; ks < BK / 16; ++ks) {
                mma_bf16(tmem + 384, desc_sw64(sa + (s - 1) * TILE_BYTES + ks * 32),
                         desc_sw64(sb + (t - 1) * TILE_BYTES + ks * 32), f_started);
                f_started = true;
              }
            }
        }
        const int c = kb / CH;
        const bool first = (kb % CH) == 0;
        if (first && c > 0) {
          if (!mbar_wait(accempty_bar, (c - 1) & 1, abort_flag)) {
            signal_abort(abort_flag);
            break;
          }
          tc_fence_after();
        }
        for (int gg = 2; gg <= gE; ++gg) {
          bool acc = !first;
          for (int s = 1; s < gg; ++s) {
            const int t = gg - s;
            if (s > S || t > S) continue;
            for (int ks = 0; ks < BK / 16; ++ks) {
              mma_bf16(tmem + (gg - 2) * 128, desc_sw64(sa + (s - 1) * TILE_BYTES + ks * 32),
                       desc_sw64(sb + (t - 1) * TILE_BYTES + ks * 32), acc);
              acc = true;
            }
          }
        }
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
      for (int gg = 2; gg <= gE; ++gg) {
        const float up = __int_as_float((127 + 7 * gg) << 23);  // 2^(7 g)
        const int sh = 7 * (gE - gg);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          uint32_t v[16];
          tmem_ld16(lbase + (uint32_t)((gg - 2) * 128 + h * 16), v);
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const float f = fmaf(__uint_as_float(v[j]), up, MAGIC);
            const long long iv = (long long)(__float_as_int(f) - MAGIC_BITS);
            R[h * 16 + j] += (long long)((unsigned long long)iv << sh);
          }
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
      const int ea = (i < g.M) ? a.expA[(long long)bz * g.M + i] : 0;
      double* Cb = g.C + (long long)bz * g.c_sb;
      const long long ri = (i < g.M) ? g.c_r.at(i) : 0;
      const bool mirror_rc = (g.sym == SYM_ROWCOL) && (m0 != n0);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        uint32_t v[16];
        if (has_inexact) {
          tmem_ld16(lbase + 384u + (uint32_t)(h * 16), v);
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = 0u;
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int jj = n0 + cg * 32 + h * 16 + j;
          if (i >= g.M || jj >= g.N) continue;
          const float t = __uint_as_float(v[j]) * upE;
          const float th = rintf(t);
          const long long hi = __float2ll_rn(th);
          const long long lo = __float2ll_rn((t - th) * upF);
          const long long z = (long long)((unsigned long long)(R[h * 16 + j] + hi) << a.frac) + lo;
          const int eb = a.expB[(long long)bz * g.N + jj];
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
using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int get_encode(EncodeFn* out) {
  static std::mutex mu;
  static EncodeFn fn = nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
    GB_REQUIRE(e == cudaSuccess && q == cudaDriverEntryPointSuccess && p, GB_ERR_CUDA,
               "cuTensorMapEncodeTiled unavailable (%s)", cudaGetErrorString(e));
    fn = reinterpret_cast<EncodeFn>(p);
  }
  *out = fn;
  return GB_OK;
}

int make_map(const SlicedDesc& d, CUtensorMap* map) {
  EncodeFn enc;
  GB_TRY(get_encode(&enc));
  GB_REQUIRE((reinterpret_cast<uintptr_t>(d.planes) & 15) == 0, GB_ERR_INVALID_ARG, "slice planes not 16-byte aligned");
  cuuint64_t dims[3] = {(cuuint64_t)d.K, (cuuint64_t)d.rows, (cuuint64_t)d.batch * d.S};
  cuuint64_t strides[2] = {(cuuint64_t)d.kpad * 2, (cuuint64_t)d.rows * d.kpad * 2};
  cuuint32_t box[3] = {BK, BM, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, d.planes, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  GB_REQUIRE(r == CUDA_SUCCESS, GB_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d) dims %llu x %llu x %llu", (int)r,
             (unsigned long long)dims[0], (unsigned long long)dims[1], (unsigned long long)dims[2]);
  return GB_OK;
}

size_t smem_bytes(int S) { return (size_t)STAGES * 2 * S * TILE_BYTES + 256 + 1024; }

}  // namespace

int ozaki_gemm(const SlicedDesc& A, const SlicedDesc& B, const OzGemm& g, cudaStream_t stream) {
  if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return GB_OK;
  GB_REQUIRE(g.S >= 1 && g.S <= 6 && A.S == g.S && B.S == g.S, GB_ERR_INVALID_ARG, "ozaki_gemm: nslices mismatch");
  GB_REQUIRE(A.rows == g.M && B.rows == g.N && A.K == g.K && B.K == g.K && A.batch == g.batch &&
                 B.batch == g.batch,
             GB_ERR_BAD_SHAPE, "ozaki_gemm: operand shapes do not match the GEMM");
  GB_REQUIRE(g.sym != SYM_ROWCOL || g.M == g.N, GB_ERR_BAD_SHAPE, "ozaki_gemm: SYM_ROWCOL needs M == N");
  GB_REQUIRE(g.sym != SYM_PAIRCOL || (long long)g.pair_n * g.pair_n == g.N, GB_ERR_BAD_SHAPE,
             "ozaki_gemm: SYM_PAIRCOL needs N == pair_n^2");
  const long long gy = (g.M + BM - 1) / BM, gx = (g.N + BN - 1) / BN;
  GB_REQUIRE(gy <= 65535 && g.batch <= 65535 && gx <= 2147483647LL, GB_ERR_BAD_SHAPE, "ozaki_gemm: grid too large");
  if (g.K == 0) {
    GB_REQUIRE(false, GB_ERR_BAD_SHAPE, "ozaki_gemm: K == 0");
  }
  CUtensorMap ma, mb;
  GB_TRY(make_map(A, &ma));
  GB_TRY(make_map(B, &mb));
  const size_t smem = smem_bytes(g.S);
  static std::mutex mu;
  static int configured_dev[64] = {0};
  {
    int dev = 0;
    GB_TRY(cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 64 && !configured_dev[dev]) {
      GB_TRY(cuda_status(cudaFuncSetAttribute(ozaki_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem_bytes(6)),
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
  KArgs ka{g, A.exps, B.exps, frac};
  dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)g.batch);
  const int pi = prof_begin(g.tag, stream);
  ozaki_kernel<<<grid, THREADS, smem, stream>>>(ma, mb, ka);
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
  cudaError_t e = cudaFuncGetAttributes(&fa, ozaki_kernel);
  int occ = -1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ozaki_kernel, THREADS, smem_bytes(6));
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
