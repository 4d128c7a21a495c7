// FP64 DMMA contraction engine: see gemm_f64.cuh for the operand model.
//
// CTA tile 64 x 64 x 16, 4 warps in a 2 x 2 arrangement, each warp owning a
// 32 x 32 block as 4 x 4 DMMA m8n8k4 tiles.  Global -> register prefetch of
// the next k-tile overlaps the DMMAs on the current shared-memory buffer
// (two buffers, one barrier per k-tile).  The loader thread map follows the
// operand's unit-stride index so that global loads coalesce.
#include "gemm_f64.cuh"

namespace gb {
namespace {

constexpr int BM = 64, BN = 64, BKT = 16, THREADS = 128, PAD = 8;

__device__ __forceinline__ void dmma(double& c0, double& c1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(c0), "+d"(c1)
               : "d"(a), "d"(b));
}

// Loader for one operand tile of R rows (the non-K index) x BKT (the K index).
// KFAST: consecutive threads take consecutive k (16 k x 8 rows per pass);
// otherwise consecutive threads take consecutive rows (64 rows x 2 k per pass).
template <bool KFAST>
struct TileLoader {
  long long off[8];   // per-slot offset of the non-K index (KFAST) or of k (!KFAST), filled per use
  bool ok[8];
  int lane_k, lane_r;

  __device__ void init(const Index2& rmap, int r0, int rlim) {
    const int tid = threadIdx.x;
    if (KFAST) {
      lane_k = tid & 15;
      lane_r = tid >> 4;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        int r = r0 + lane_r + 8 * i;
        ok[i] = r < rlim;
        off[i] = ok[i] ? rmap.at(r) : 0;
      }
    } else {
      lane_r = tid & 63;
      lane_k = tid >> 6;
      int r = r0 + lane_r;
      ok[0] = r < rlim;
      off[0] = ok[0] ? rmap.at(r) : 0;
    }
  }

  // Load the k-tile starting at k0 into v[8].
  __device__ void load(const double* __restrict__ base, const Index2& kmap, int k0, int klim,
                       double (&v)[8]) const {
    if (KFAST) {
      int k = k0 + lane_k;
      bool kok = k < klim;
      long long ko = kok ? kmap.at(k) : 0;
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = (kok && ok[i]) ? __ldg(base + off[i] + ko) : 0.0;
    } else {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        int k = k0 + lane_k + 2 * i;
        bool kok = k < klim && ok[0];
        v[i] = kok ? __ldg(base + off[0] + kmap.at(k)) : 0.0;
      }
    }
  }

  // Store v[8] into smem laid out as S[k][row] (row-contiguous).
  template <int LD>
  __device__ void store(double (*S)[LD], const double (&v)[8]) const {
    if (KFAST) {
#pragma unroll
      for (int i = 0; i < 8; ++i) S[lane_k][lane_r + 8 * i] = v[i];
    } else {
#pragma unroll
      for (int i = 0; i < 8; ++i) S[lane_k + 2 * i][lane_r] = v[i];
    }
  }
};

template <bool AK, bool BKF>
__global__ void __launch_bounds__(THREADS) gemm_f64_kernel(const GemmF64 g) {
  __shared__ double As[2][BKT][BM + PAD];
  __shared__ double Bs[2][BKT][BN + PAD];

  const int m0 = blockIdx.y * BM;
  const int n0 = blockIdx.x * BN;
  const long long bz = blockIdx.z;

  if (g.sym == SYM_ROWCOL && m0 > n0) return;
  if (g.sym == SYM_PAIRCOL) {
    const int j1 = min(n0 + BN, g.N) - 1;
    const int ma = n0 / g.pair_n, mb = j1 / g.pair_n;
    if (ma == mb && (j1 % g.pair_n) < ma) return;
  }

  const double* __restrict__ Ab = g.A.p + bz * g.A.sb;
  const double* __restrict__ Bb = g.B.p + bz * g.B.sb;

  TileLoader<AK> la;
  TileLoader<BKF> lb;
  la.init(g.A.r, m0, g.M);   // A rows are the M index, A columns the K index
  lb.init(g.B.c, n0, g.N);   // B columns are the N index, B rows the K index

  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int wm = warp >> 1, wn = warp & 1;
  const int gq = lane >> 2, tq = lane & 3;

  double acc[4][4][2];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b][0] = acc[a][b][1] = 0.0;

  double va[8], vb[8];
  const int nk = (g.K + BKT - 1) / BKT;
  if (nk > 0) {
    la.load(Ab, g.A.c, 0, g.K, va);
    lb.load(Bb, g.B.r, 0, g.K, vb);
    la.template store<BM + PAD>(As[0], va);
    lb.template store<BN + PAD>(Bs[0], vb);
  }
  __syncthreads();

  for (int kt = 0; kt < nk; ++kt) {
    const int cur = kt & 1;
    const bool more = kt + 1 < nk;
    if (more) {
      la.load(Ab, g.A.c, (kt + 1) * BKT, g.K, va);
      lb.load(Bb, g.B.r, (kt + 1) * BKT, g.K, vb);
    }
#pragma unroll
    for (int ks = 0; ks < BKT / 4; ++ks) {
      double af[4], bf[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        af[t] = As[cur][ks * 4 + tq][wm * 32 + t * 8 + gq];
        bf[t] = Bs[cur][ks * 4 + tq][wn * 32 + t * 8 + gq];
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) dmma(acc[a][b][0], acc[a][b][1], af[a], bf[b]);
    }
    if (more) {
      la.template store<BM + PAD>(As[cur ^ 1], va);
      lb.template store<BN + PAD>(Bs[cur ^ 1], vb);
    }
    __syncthreads();
  }

  double* __restrict__ Cb = g.C.p + bz * g.C.sb;
  const bool mirror_rc = (g.sym == SYM_ROWCOL) && (m0 != n0);
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int i = m0 + wm * 32 + a * 8 + gq;
    if (i >= g.M) continue;
    const long long ri = g.C.r.at(i);
#pragma unroll
    for (int b = 0; b < 4; ++b) {
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int j = n0 + wn * 32 + b * 8 + 2 * tq + e;
        if (j >= g.N) continue;
        double v = g.alpha * acc[a][b][e];
        double* dst = Cb + ri + g.C.c.at(j);
        if (g.beta != 0.0) v += g.beta * *dst;
        *dst = v;
        if (mirror_rc) {
          Cb[g.C.r.at(j) + g.C.c.at(i)] = v;
        } else if (g.sym == SYM_PAIRCOL) {
          const int mm = j / g.pair_n, nn = j % g.pair_n;
          if (nn > mm) Cb[ri + g.C.c.at((long long)nn * g.pair_n + mm)] = v;
        }
      }
    }
  }
}

// Small outputs: one warp per 8 x 8 block of C, DMMA m8n8k4 straight from
// global memory (operands of small GEMMs sit in L2), loads batched UNR k-steps
// ahead.  GB300's FP64 rate per SM is low (~7 GFLOP/s), so a GEMM that gives
// the 64 x 64 kernel fewer CTAs than SMs is latency-bound on a few SMs; 8 x 8
// blocks spread it over the whole GPU.
template <int UNR>
__global__ void __launch_bounds__(32) gemm_f64_small_kernel(const GemmF64 g) {
  const int lane = threadIdx.x;
  const int m0 = blockIdx.y * 8, n0 = blockIdx.x * 8;
  const long long bz = blockIdx.z;
  if (g.sym == SYM_ROWCOL && m0 > n0) return;
  if (g.sym == SYM_PAIRCOL) {
    const int j1 = min(n0 + 8, g.N) - 1;
    const int ma = n0 / g.pair_n, mb = j1 / g.pair_n;
    if (ma == mb && (j1 % g.pair_n) < ma) return;
  }
  const int gq = lane >> 2, tq = lane & 3;
  const int ia = m0 + gq, jb = n0 + gq;  // A row / B column of this lane's fragments
  const bool iok = ia < g.M, jok = jb < g.N;
  const double* __restrict__ Ab = g.A.p + bz * g.A.sb + (iok ? g.A.r.at(ia) : 0);
  const double* __restrict__ Bb = g.B.p + bz * g.B.sb + (jok ? g.B.c.at(jb) : 0);
  double c0 = 0.0, c1 = 0.0;
  for (int k0 = 0; k0 < g.K; k0 += 4 * UNR) {
    double a[UNR], b[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      const int k = k0 + 4 * u + tq;
      const bool kok = k < g.K;
      a[u] = (iok && kok) ? __ldg(Ab + g.A.c.at(k)) : 0.0;
      b[u] = (jok && kok) ? __ldg(Bb + g.B.r.at(k)) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < UNR; ++u) dmma(c0, c1, a[u], b[u]);
  }
  double* __restrict__ Cb = g.C.p + bz * g.C.sb;
  const int i = m0 + gq;
  if (i >= g.M) return;
  const bool mirror_rc = (g.sym == SYM_ROWCOL) && (m0 != n0);
  const long long ri = g.C.r.at(i);
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    const int j = n0 + 2 * tq + e;
    if (j >= g.N) continue;
    if (g.sym == SYM_ROWCOL && m0 == n0 && j < i) continue;  // the diagonal block's mirror writes these
    double v = g.alpha * (e ? c1 : c0);
    double* dst = Cb + ri + g.C.c.at(j);
    if (g.beta != 0.0) v += g.beta * *dst;
    *dst = v;
    if (g.sym == SYM_ROWCOL && (mirror_rc || j > i)) {
      Cb[g.C.r.at(j) + g.C.c.at(i)] = v;
    } else if (g.sym == SYM_PAIRCOL) {
      const int mm = j / g.pair_n, nn = j % g.pair_n;
      if (nn > mm) Cb[ri + g.C.c.at((long long)nn * g.pair_n + mm)] = v;
    }
  }
}

}  // namespace

int gemm_f64(const GemmF64& g, cudaStream_t stream) {
  if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return GB_OK;
  GB_REQUIRE(g.K >= 0, GB_ERR_BAD_SHAPE, "gemm_f64: negative K");
  GB_REQUIRE(g.sym == SYM_NONE || g.beta == 0.0, GB_ERR_INVALID_ARG,
             "gemm_f64: symmetric modes do not take beta");
  GB_REQUIRE(g.sym != SYM_ROWCOL || g.M == g.N, GB_ERR_BAD_SHAPE, "gemm_f64: SYM_ROWCOL needs M == N");
  GB_REQUIRE(g.sym != SYM_PAIRCOL || (g.pair_n > 0 && (long long)g.pair_n * g.pair_n == g.N),
             GB_ERR_BAD_SHAPE, "gemm_f64: SYM_PAIRCOL needs N == pair_n^2");
  const long long gy = (g.M + BM - 1) / BM;
  const long long gx = (g.N + BN - 1) / BN;
  GB_REQUIRE(gy <= 65535 && g.batch <= 65535 && gx <= 2147483647LL, GB_ERR_BAD_SHAPE,
             "gemm_f64: grid too large (M=%d N=%d batch=%d)", g.M, g.N, g.batch);
  if (gx * gy * g.batch < 152 && g.M <= 65535 * 8) {
    // fewer 64 x 64 tiles than SMs: spread 8 x 8 blocks over the GPU instead
    const dim3 sgrid((unsigned)((g.N + 7) / 8), (unsigned)((g.M + 7) / 8), (unsigned)g.batch);
    GB_LAUNCH(g.tag, stream, gemm_f64_small_kernel<4><<<sgrid, 32, 0, stream>>>(g));
    return GB_OK;
  }
  dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)g.batch);
  if (g.a_kfast && g.b_kfast)
    GB_LAUNCH(g.tag, stream, gemm_f64_kernel<true, true><<<grid, THREADS, 0, stream>>>(g));
  else if (g.a_kfast)
    GB_LAUNCH(g.tag, stream, gemm_f64_kernel<true, false><<<grid, THREADS, 0, stream>>>(g));
  else if (g.b_kfast)
    GB_LAUNCH(g.tag, stream, gemm_f64_kernel<false, true><<<grid, THREADS, 0, stream>>>(g));
  else
    GB_LAUNCH(g.tag, stream, gemm_f64_kernel<false, false><<<grid, THREADS, 0, stream>>>(g));
  return GB_OK;
}

}  // namespace gb
