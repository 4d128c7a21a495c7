// Occupation optimiser on the device: E(gamma), dE/dgamma and the whole
// conjugate-gradient minimisation over gamma at fixed J_MO, K_MO, H_core
// (occoptr, minimization.py:77-97, which calls scipy's CG on calcocce /
// calcoccg), without a host round trip per evaluation.
//
// One evaluation at a trial point gamma_t:
//  - occupations from the softmax parameterisation (ocupacion_softmax,
//    pnof.py:770-809; the strong occupation of pair i written at index i as
//    the reference does) and the per-orbital GNOF quantities of CJCKD8
//    (pnof.py:350-422): n, nd = n F(n_s), sqrt(nd), fi = sqrt(n (1 - n)) and
//    its derivative;
//  - the pair sums over (a, b) from different pairs (calce, pnof.py:905-929,
//    and the gradient of calcoccg, pnof.py:1004-1033 with der_CJCKD8,
//    pnof.py:425-525): occ_rows_kernel, one warp per (32 orbitals a, 16
//    orbitals b) item, lanes over a so that J[b][a] and K[b][a] are read
//    coalesced.  The terms of a are linear in five weighted sums over b
//    (n_b J_ba, n_b K_ba, and over the dynamic / static pairs fi_b K_ba,
//    +-nd12_b K_ba, nd_b K_ba): at most five FMAs per pair.  The last warp to
//    finish an a-group (an atomic count per group, no waiting) adds the
//    group's items;
//  - occ_step_kernel (one CTA): the diagonal and same-pair terms, the chain
//    rule through nd = n F(n_s), g = dn^T e, and the energy -- the assembly
//    of the host loop of occ_host.cu, summed in pairwise trees.
//
// GB300's FP64 unit has a long dependent latency (~64 clocks for an add or
// FMA, several hundred for a division or square root, ~1000 for exp), so the
// kernels are laid out for short FP64 dependency chains and few FP64
// operations: every exponential of a trial point in its own thread, the pair
// loop unrolled with masks into interleaved FMA chains, tree sums, and the
// conjugate-gradient scalars of one evaluation from one
// fused block reduction (the next search's g.g and g.p follow from it
// algebraically).
//
// The minimiser is scipy's CG as scipy 1.18 runs it: Polak-Ribiere+ with the
// sufficient-descent check, the first trial step from the previous decrease,
// and the line search of More & Thuente (ACM TOMS 20 (1994) 286-307; strong
// Wolfe with c1 = 1e-4, c2 = 0.4, xtol 1e-14, steps in [1e-100, 1e100], at most
// 100 calls), as a state machine that occ_step_kernel advances by one
// evaluation.  Where scipy would try its second line search (a failed search,
// or a step without sufficient descent), the state machine restarts from
// steepest descent once and otherwise stops at the current point.
//
// One CUDA graph per workspace runs a whole minimisation: an init kernel, a
// WHILE conditional node whose body is four rounds of rows -> step (the step
// kernel clears the condition when the minimiser stops and the kernels after
// it return at once), then the occupations and C^J, C^K at the result.  The
// number of evaluations is capped at 1 + 200 (maxiter + 1): a minimiser that
// reaches the cap reports success -1.  The host-driven form
// (gb_occ_minimize_dev_sync) replays an ordinary graph of eight rounds instead
// of the conditional node and reads the phase back after each replay.
//
// All arithmetic is FP64 (GB300's FP64 rate is low, so the O(nbf5^2) pair
// work is spread over the whole GPU and the single-CTA work is O(nbf5)).
// Closed shell without singly occupied orbitals (MSpin = 0, nsoc = 0).
#include <cmath>
#include <cstddef>
#include <map>
#include <mutex>
#include <tuple>

#include "gb_common.cuh"

namespace {

constexpr int kStepThreads = 256;  // one-CTA kernels
constexpr int kMinBlocks = 1;
constexpr int kRowCtas = 4 * 152;  // rows kernel: one warp per CTA, grid-stride over items
constexpr int kUnroll = 4;         // evaluations per round of the WHILE node
constexpr int kCjckCtas = 2 * 152;
constexpr int kBch = 16;           // orbitals b per item of the rows kernel
constexpr double kHCut = 0.02 * 1.4142135623730951;
// line search constants
constexpr double kFtol = 1e-4, kGtol = 0.4, kXtol = 1e-14, kStpMin = 1e-100, kStpMax = 1e100;
constexpr double kXtrapL = 1.1, kXtrapU = 4.0, kP5 = 0.5, kP66 = 0.66;
constexpr int kMaxCalls = 100;

enum { MODE_MIN = 0, MODE_EVAL = 1 };
enum { PH_INIT = 0, PH_LS = 1, PH_DONE = 2 };
enum { T_FG = 0, T_CONV = 1, T_FAIL = 2 };

struct OccArgs {
  const double *J, *K, *H, *gamma0;
  double *gamma_out, *grad_out, *res, *n_out, *cj_out, *ck_out;
  // workspace arrays
  double *x, *g, *p, *pn, *xt, *gt;             // nv
  double *n, *nd, *nd12, *fi, *fid, *sq, *rsq;  // P
  double *e, *en;                               // P
  double *ns, *F, *dF;                          // ndoc
  double *nw;                                   // nv
  double *part;                                 // 5 P nbc (per item: A1 .. A5)
  double *row;                                  // 5 P (per orbital, all items)
  int *pair_of, *cls;                           // P
  unsigned int* grp;                            // per a-group: items done
  int P, no1, ndoc, ncwo, nv, nbc, maxiter, mode;
  double gtol;
};

struct OccState {
  OccArgs a;
  // conjugate gradients (delta = g.g, d0 = g.p of the next line search)
  double f, f_prev, gnorm, delta, d0;
  int k, nev, maxev, phase, restarted;
  // More-Thuente line search
  double stp, finit, ginit, gtest, width, width1, stx, fx, gx, sty, fy, gy, stmin, stmax;
  int brackt, stage, calls;
};

__device__ __forceinline__ int weak_of(const OccArgs& a, int p, int j) {
  return a.no1 + a.ndoc + (a.ndoc - p - 1) + a.ndoc * j;
}
__device__ __forceinline__ int gam_of(const OccArgs& a, int p, int j) { return (a.ndoc - p - 1) + a.ndoc * j; }

// NaN-propagating maximum (numpy's max)
__device__ __forceinline__ double nanmax(double a, double b) { return (a > b || a != a) ? a : b; }

// ---- deterministic block reductions (fixed tree; every thread gets the
// values): NS sums and, with MAX, a NaN-propagating maximum in slot NS
template <int NS, bool MAX>
__device__ void block_reduce(double (&v)[NS + (MAX ? 1 : 0)], double* sh) {
  constexpr int NV = NS + (MAX ? 1 : 0);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const double y = __shfl_down_sync(0xffffffffu, v[q], o);
      v[q] = (MAX && q == NS) ? nanmax(v[q], y) : v[q] + y;
    }
  }
  __syncthreads();
  if (l == 0)
#pragma unroll
    for (int q = 0; q < NV; ++q) sh[q * 8 + w] = v[q];
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = l < kStepThreads / 32 ? sh[q * 8 + l] : 0.0;
    for (int o = 4; o > 0; o >>= 1) {
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        const double y = __shfl_down_sync(0xffffffffu, v[q], o);
        v[q] = (MAX && q == NS) ? nanmax(v[q], y) : v[q] + y;
      }
    }
    if (l == 0)
#pragma unroll
      for (int q = 0; q < NV; ++q) sh[64 + q] = v[q];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = sh[64 + q];
  __syncthreads();
}

// ---- the trial point's per-orbital quantities (all threads of one CTA)
__device__ void prep_point(const OccArgs& a, const double* __restrict__ x) {
  const int tid = threadIdx.x, nd = a.ndoc, nc = a.ncwo;
  // one exponential per logit, all at once (a pair with a logit past exp's
  // range is redone with its largest logit below)
  for (int t = tid; t < a.nv; t += kStepThreads) {
    const int j = t / nd, p = nd - 1 - (t - j * nd);  // t = gam_of(p, j)
    a.nw[p * nc + j] = exp(fmin(x[t], 700.0));
  }
  __syncthreads();
  for (int p = tid; p < nd; p += kStepThreads) {
    double top = -INFINITY;
    for (int j = 0; j < nc; ++j) top = fmax(top, x[gam_of(a, p, j)]);
    double* w = a.nw + p * nc;
    double ns;
    if (top >= 700.0) {
      // logits past exp's range: the same softmax shifted by the largest one
      double den = exp(-top);
      for (int j = 0; j < nc; ++j) den += exp(x[gam_of(a, p, j)] - top);
      ns = exp(-top) / den;
      for (int j = 0; j < nc; ++j) w[j] = exp(x[gam_of(a, p, j)] - top) / den;
    } else {
      double den = 1.0;
      for (int j = 0; j < nc; ++j) den += w[j];
      ns = 1.0 / den;
      for (int j = 0; j < nc; ++j) w[j] = w[j] / den;
    }
    a.ns[p] = ns;
    a.n[p] = ns;
    for (int j = 0; j < nc; ++j) a.n[weak_of(a, p, j)] = w[j];
  }
  __syncthreads();
  for (int p = tid; p < nd; p += kStepThreads) {
    const int s = a.no1 + p;
    const double coc = (1.0 - a.n[s]) / kHCut;
    const double F = exp(-coc * coc);
    a.F[p] = F;
    a.dF[p] = 2.0 * coc / kHCut;  // (1/F) dF/dn_s
    a.nd[s] = a.n[s] * F;
    for (int j = 0; j < nc; ++j) {
      const int w = weak_of(a, p, j);
      a.nd[w] = a.n[w] * F;
    }
  }
  __syncthreads();
  for (int i = tid; i < a.P; i += kStepThreads) {
    const double ni = a.n[i];
    const double fi = sqrt(fmax(ni * (1.0 - ni), 0.0));
    const double sq = sqrt(ni);
    a.nd12[i] = sqrt(a.nd[i]);
    a.fi[i] = fi;
    a.fid[i] = i < a.no1 ? 0.0 : (1.0 - 2.0 * ni) / (2.0 * fmax(fi, 1e-15));
    a.sq[i] = sq;
    a.rsq[i] = ni >= 1e-15 ? 1.0 / sq : 1.0 / sqrt(1e-15);
  }
  __syncthreads();
}

// ---- per orbital a, five weighted sums over the orbitals b of other pairs:
// A1 = sum n_b J_ba, A2 = sum n_b K_ba and, over the pairs with the GNOF
// dynamic / static terms (a strong and b weak, or a weak and b not core),
// A3 = sum fi_b K_ba, A4 = sum s_ab nd12_b K_ba (s = -1 weak-weak),
// A5 = sum nd_b K_ba.  The energy and gradient terms of a are linear in them
// (assemble).  The last warp of an a-group adds the group's items.
__global__ void __launch_bounds__(32) occ_rows_kernel(const OccState* __restrict__ st) {
  const OccArgs& a = st->a;
  if (st->phase == PH_DONE) return;
  const int P = a.P, nbc = a.nbc, lane = threadIdx.x;
  const int nag = (P + 31) / 32;
  const size_t plane = (size_t)P * nbc;
  for (int it = blockIdx.x; it < nag * nbc; it += gridDim.x) {
    const int ag = it / nbc, bc = it - ag * nbc;
    const int i = ag * 32 + lane;
    const bool live = i < P;
    const int ii = live ? i : P - 1;
    const int pa = a.pair_of[ii], ca = a.cls[ii];
    // two interleaved FMA chains per sum (even / odd b)
    double s1[2] = {0.0, 0.0}, s2[2] = {0.0, 0.0}, s3[2] = {0.0, 0.0}, s4[2] = {0.0, 0.0}, s5[2] = {0.0, 0.0};
    const int b0 = bc * kBch;
#pragma unroll
    for (int u = 0; u < kBch; ++u) {
      const int b = min(b0 + u, P - 1);
      const bool ok = b0 + u < P && b != ii && !(pa >= 0 && a.pair_of[b] == pa);
      const double Jba = a.J[(size_t)b * P + ii], Kba = a.K[(size_t)b * P + ii];
      const int cb = a.cls[b];
      const double wn = ok ? a.n[b] : 0.0;
      const bool chi = ok && ((ca == 1 && cb == 2) || (ca == 2 && cb >= 1));
      const double sg = (ca == 2 && cb == 2) ? -1.0 : 1.0;
      s1[u & 1] = fma(wn, Jba, s1[u & 1]);
      s2[u & 1] = fma(wn, Kba, s2[u & 1]);
      s3[u & 1] = fma(chi ? a.fi[b] : 0.0, Kba, s3[u & 1]);
      s4[u & 1] = fma(chi ? sg * a.nd12[b] : 0.0, Kba, s4[u & 1]);
      s5[u & 1] = fma(chi ? a.nd[b] : 0.0, Kba, s5[u & 1]);
    }
    double* q = a.part + (size_t)ii * nbc + bc;
    if (live) {
      q[0] = s1[0] + s1[1];
      q[plane] = s2[0] + s2[1];
      q[2 * plane] = s3[0] + s3[1];
      q[3 * plane] = s4[0] + s4[1];
      q[4 * plane] = s5[0] + s5[1];
    }
    // the last of the group's nbc items adds them up (the counter is left at
    // zero for the next evaluation)
    __threadfence();
    __syncwarp();  // every lane's partials are visible before the count moves
    unsigned int done = 0;
    if (lane == 0) done = atomicAdd(a.grp + ag, 1u);
    done = __shfl_sync(0xffffffffu, done, 0);
    if (done == (unsigned int)nbc - 1) {
      __threadfence();
      if (live) {
        const double* r = a.part + (size_t)i * nbc;
        double t[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        for (int c = 0; c < nbc; ++c)
#pragma unroll
          for (int k = 0; k < 5; ++k) t[k] += __ldcg(r + k * plane + c);
#pragma unroll
        for (int k = 0; k < 5; ++k) a.row[k * P + i] = t[k];
      }
      if (lane == 0) a.grp[ag] = 0;
    }
  }
}

// ---- energy and gradient at the trial point from the orbitals' sums (one CTA)
__device__ double assemble(const OccArgs& a, double* sh) {
  const int P = a.P, tid = threadIdx.x;
  double es = 0.0;
  for (int i = tid; i < P; i += kStepThreads) {
    const double d = 2.0 * a.H[i] + a.J[(size_t)i * P + i];
    const double A1 = a.row[i], A2 = a.row[P + i], A3 = a.row[2 * P + i], A4 = a.row[3 * P + i],
                 A5 = a.row[4 * P + i];
    const double ni = a.n[i];
    // pairs (i, b), b of another pair: sum_b 2 n_i n_b J_bi - C^K_ib K_bi
    es += ni * d + (2.0 * ni * A1 - ni * A2 - a.fi[i] * A3 - a.nd12[i] * A4 + a.nd[i] * A5);
    a.e[i] = d + 4.0 * A1 - 2.0 * A2 - 2.0 * a.fid[i] * A3;
    a.en[i] = -2.0 * (A4 / (2.0 * fmax(a.nd12[i], 1e-15)) - A5);
  }
  __syncthreads();
  // pairs inside one pair block: C^J = 0; C^K = sqrt(n_s n_w) (strong-weak),
  // -sqrt(n_w n_w') (weak-weak)
  for (int p = tid; p < a.ndoc; p += kStepThreads) {
    const int s = a.no1 + p;
    double e_s = a.e[s], ep = 0.0;
    for (int j = 0; j < a.ncwo; ++j) {
      const int w = weak_of(a, p, j);
      const double Kws = a.K[(size_t)w * P + s], Ksw = a.K[(size_t)s * P + w];
      double ew = 0.0, ej = -(a.sq[s] * a.sq[w]) * (Kws + Ksw);
      e_s -= a.sq[w] * a.rsq[s] * Kws;
      for (int j2 = 0; j2 < a.ncwo; ++j2) {
        if (j2 == j) continue;
        const int w2 = weak_of(a, p, j2);
        const double Kw2w = a.K[(size_t)w2 * P + w];
        ej += a.sq[w] * a.sq[w2] * Kw2w;
        ew += a.sq[w2] * Kw2w;
      }
      ep += ej;
      a.e[w] = a.e[w] - a.sq[s] * a.rsq[w] * Ksw + a.rsq[w] * ew;
    }
    a.e[s] = e_s;
    es += ep;
  }
  __syncthreads();
  // nd_s = n_s F(n_s), nd_w = n_w F(n_s): chain dE/dnd to the occupations
  for (int p = tid; p < a.ndoc; p += kStepThreads) {
    const int s = a.no1 + p;
    const double F = a.F[p], dF = a.dF[p];
    double e_s = a.e[s] + a.en[s] * F * (1.0 + a.n[s] * dF);
    for (int j = 0; j < a.ncwo; ++j) {
      const int w = weak_of(a, p, j);
      a.e[w] += a.en[w] * F;
      e_s += a.en[w] * a.n[w] * F * dF;
    }
    a.e[s] = e_s;
  }
  __syncthreads();
  // g = dn^T e (row p of dn holds the strong occupation)
  for (int p = tid; p < a.ndoc; p += kStepThreads) {
    double wsum = 0.0;
    for (int i = 0; i < a.ncwo; ++i) wsum += a.nw[p * a.ncwo + i] * a.e[weak_of(a, p, i)];
    for (int j = 0; j < a.ncwo; ++j) {
      const double w = a.nw[p * a.ncwo + j];
      a.gt[gam_of(a, p, j)] = -a.ns[p] * w * a.e[p] + w * a.e[weak_of(a, p, j)] - w * wsum;
    }
  }
  double v[1] = {es};
  block_reduce<1, false>(v, sh);  // synchronises
  return v[0];
}

// ---- More & Thuente, one safeguarded step (section 4 of the paper)
__device__ void dcstep(double& stx, double& fx, double& dx, double& sty, double& fy, double& dy, double& stp,
                       double fp, double dp, int& brackt, double stpmin, double stpmax) {
  const double sgnd = dp * (dx / fabs(dx));
  double stpf;
  if (fp > fx) {
    const double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
    const double s = fmax(fmax(fabs(theta), fabs(dx)), fabs(dp));
    double gamma = s * sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
    if (stp < stx) gamma = -gamma;
    const double p = (gamma - dx) + theta;
    const double q = ((gamma - dx) + gamma) + dp;
    const double r = p / q;
    const double stpc = stx + r * (stp - stx);
    const double stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2.0) * (stp - stx);
    stpf = fabs(stpc - stx) < fabs(stpq - stx) ? stpc : stpc + (stpq - stpc) / 2.0;
    brackt = 1;
  } else if (sgnd < 0.0) {
    const double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
    const double s = fmax(fmax(fabs(theta), fabs(dx)), fabs(dp));
    double gamma = s * sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
    if (stp > stx) gamma = -gamma;
    const double p = (gamma - dp) + theta;
    const double q = ((gamma - dp) + gamma) + dx;
    const double r = p / q;
    const double stpc = stp + r * (stx - stp);
    const double stpq = stp + (dp / (dp - dx)) * (stx - stp);
    stpf = fabs(stpc - stp) > fabs(stpq - stp) ? stpc : stpq;
    brackt = 1;
  } else if (fabs(dp) < fabs(dx)) {
    const double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
    const double s = fmax(fmax(fabs(theta), fabs(dx)), fabs(dp));
    const double disc = (theta / s) * (theta / s) - (dx / s) * (dp / s);
    double gamma = s * sqrt(disc > 0.0 ? disc : 0.0);
    if (stp > stx) gamma = -gamma;
    const double p = (gamma - dp) + theta;
    const double q = (gamma + (dx - dp)) + gamma;
    const double r = p / q;
    double stpc;
    if (r < 0.0 && gamma != 0.0)
      stpc = stp + r * (stx - stp);
    else if (stp > stx)
      stpc = stpmax;
    else
      stpc = stpmin;
    const double stpq = stp + (dp / (dp - dx)) * (stx - stp);
    if (brackt) {
      stpf = fabs(stpc - stp) < fabs(stpq - stp) ? stpc : stpq;
      if (stp > stx)
        stpf = fmin(stp + kP66 * (sty - stp), stpf);
      else
        stpf = fmax(stp + kP66 * (sty - stp), stpf);
    } else {
      stpf = fabs(stpc - stp) > fabs(stpq - stp) ? stpc : stpq;
      stpf = fmin(stpmax, stpf);
      stpf = fmax(stpmin, stpf);
    }
  } else {
    if (brackt) {
      const double theta = 3.0 * (fp - fy) / (sty - stp) + dy + dp;
      const double s = fmax(fmax(fabs(theta), fabs(dy)), fabs(dp));
      double gamma = s * sqrt((theta / s) * (theta / s) - (dy / s) * (dp / s));
      if (stp > sty) gamma = -gamma;
      const double p = (gamma - dp) + theta;
      const double q = ((gamma - dp) + gamma) + dy;
      const double r = p / q;
      stpf = stp + r * (sty - stp);
    } else if (stp > stx) {
      stpf = stpmax;
    } else {
      stpf = stpmin;
    }
  }
  if (fp > fx) {
    sty = stp;
    fy = fp;
    dy = dp;
  } else {
    if (sgnd < 0.0) {
      sty = stx;
      fy = fx;
      dy = dx;
    }
    stx = stp;
    fx = fp;
    dx = dp;
  }
  stp = stpf;
}

__device__ int ls_fg(OccState& S, double stp) {
  if (!isfinite(stp) || S.calls >= kMaxCalls) return T_FAIL;
  S.stp = stp;
  return T_FG;
}

__device__ int ls_start(OccState& S, double stp, double f, double g) {
  S.calls = 1;
  if (stp < kStpMin || stp > kStpMax || g >= 0.0) return T_FAIL;
  S.brackt = 0;
  S.stage = 1;
  S.finit = f;
  S.ginit = g;
  S.gtest = kFtol * g;
  S.width = kStpMax - kStpMin;
  S.width1 = S.width / kP5;
  S.stx = 0.0;
  S.fx = f;
  S.gx = g;
  S.sty = 0.0;
  S.fy = f;
  S.gy = g;
  S.stmin = 0.0;
  S.stmax = stp + kXtrapU * stp;
  return ls_fg(S, stp);
}

__device__ int ls_step(OccState& S, double f, double g) {
  S.calls += 1;
  double stp = S.stp;
  const double ftest = S.finit + stp * S.gtest;
  if (S.stage == 1 && f <= ftest && g >= 0.0) S.stage = 2;
  const bool warn = (S.brackt && (stp <= S.stmin || stp >= S.stmax)) ||
                    (S.brackt && S.stmax - S.stmin <= kXtol * S.stmax) ||
                    (stp == kStpMax && f <= ftest && g <= S.gtest) ||
                    (stp == kStpMin && (f > ftest || g >= S.gtest));
  if (f <= ftest && fabs(g) <= kGtol * (-S.ginit)) return T_CONV;
  if (warn) return T_FAIL;
  if (S.stage == 1 && f <= S.fx && f > ftest) {
    // the modified function psi(a) = phi(a) - phi(0) - ftol phi'(0) a
    double fxm = S.fx - S.stx * S.gtest, fym = S.fy - S.sty * S.gtest;
    double gxm = S.gx - S.gtest, gym = S.gy - S.gtest;
    dcstep(S.stx, fxm, gxm, S.sty, fym, gym, stp, f - stp * S.gtest, g - S.gtest, S.brackt, S.stmin, S.stmax);
    S.fx = fxm + S.stx * S.gtest;
    S.fy = fym + S.sty * S.gtest;
    S.gx = gxm + S.gtest;
    S.gy = gym + S.gtest;
  } else {
    dcstep(S.stx, S.fx, S.gx, S.sty, S.fy, S.gy, stp, f, g, S.brackt, S.stmin, S.stmax);
  }
  if (S.brackt) {
    if (fabs(S.sty - S.stx) >= kP66 * S.width1) stp = S.stx + kP5 * (S.sty - S.stx);
    S.width1 = S.width;
    S.width = fabs(S.sty - S.stx);
    S.stmin = fmin(S.stx, S.sty);
    S.stmax = fmax(S.stx, S.sty);
  } else {
    S.stmin = stp + kXtrapL * (stp - S.stx);
    S.stmax = stp + kXtrapU * (stp - S.stx);
  }
  stp = fmin(fmax(stp, kStpMin), kStpMax);
  if ((S.brackt && (stp <= S.stmin || stp >= S.stmax)) || (S.brackt && S.stmax - S.stmin <= kXtol * S.stmax))
    stp = S.stx;
  return ls_fg(S, stp);
}

// ---- kernels
__global__ void __launch_bounds__(kStepThreads, kMinBlocks) occ_init_kernel(OccState* st, OccArgs args) {
  OccState& S = *st;
  const int tid = threadIdx.x;
  if (tid == 0) {
    S.a = args;
    S.phase = PH_INIT;
    S.nev = 0;
    S.k = 0;
    S.restarted = 0;
    S.maxev = 1 + 200 * (args.maxiter + 1);
  }
  const OccArgs& a = args;
  const int nb = a.no1 + a.ndoc;
  for (int i = tid; i < a.P; i += kStepThreads) {
    a.n[i] = 0.0;
    a.nd[i] = 0.0;
    a.pair_of[i] = -1;
    a.cls[i] = i < a.no1 ? 0 : (i < nb ? 1 : 2);  // 1: strong set S, 2: weak set W
  }
  __syncthreads();
  for (int g = tid; g < (a.P + 31) / 32; g += kStepThreads) a.grp[g] = 0u;
  for (int p = tid; p < a.ndoc; p += kStepThreads) {
    a.pair_of[a.no1 + p] = p;
    for (int j = 0; j < a.ncwo; ++j) a.pair_of[weak_of(a, p, j)] = p;
  }
  for (int i = tid; i < a.nv; i += kStepThreads) {
    a.x[i] = a.gamma0[i];
    a.xt[i] = a.gamma0[i];
  }
  __syncthreads();
  prep_point(a, a.xt);
}

__device__ void finish(OccState& S, double success, cudaGraphConditionalHandle h, int cond) {
  const OccArgs& a = S.a;
  for (int i = threadIdx.x; i < a.nv; i += kStepThreads) a.gamma_out[i] = a.x[i];
  if (threadIdx.x == 0) {
    a.res[0] = S.f;
    a.res[1] = S.k;
    a.res[2] = S.nev;
    a.res[3] = success;
    a.res[4] = S.gnorm;
    S.phase = PH_DONE;
    if (cond) cudaGraphSetConditional(h, 0);
  }
}

// The state word by word between global and shared memory.
__device__ __forceinline__ void copy_state(OccState* dst, const OccState* src) {
  static_assert(sizeof(OccState) % 8 == 0, "OccState in 8-byte words");
  const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
  unsigned long long* d = reinterpret_cast<unsigned long long*>(dst);
  for (int i = threadIdx.x; i < (int)(sizeof(OccState) / 8); i += blockDim.x) d[i] = s[i];
}

__device__ void step_body(OccState& S, double* sh, int& s_act, cudaGraphConditionalHandle h, int cond);

__global__ void __launch_bounds__(kStepThreads, kMinBlocks) occ_step_kernel(OccState* st, cudaGraphConditionalHandle h, int cond) {
  __shared__ double sh[72];
  __shared__ int s_act;
  // the step works on a copy in shared memory: its scalars and the array
  // pointers are read there, not from global memory behind every store
  __shared__ OccState S;
  if (st->phase == PH_DONE) {
    if (threadIdx.x == 0 && cond) cudaGraphSetConditional(h, 0);
    return;
  }
  copy_state(&S, st);
  __syncthreads();
  step_body(S, sh, s_act, h, cond);
  __syncthreads();
  copy_state(st, &S);
}

__device__ void step_body(OccState& S, double* sh, int& s_act, cudaGraphConditionalHandle h, int cond) {
  const OccArgs& a = S.a;
  const int tid = threadIdx.x;
  const double E = assemble(a, sh);
  if (tid == 0) S.nev += 1;
  if (a.mode == MODE_EVAL) {
    double v[1] = {0.0};
    for (int i = tid; i < a.nv; i += kStepThreads) {
      if (a.grad_out) a.grad_out[i] = a.gt[i];
      a.x[i] = a.xt[i];
      v[0] = nanmax(v[0], fabs(a.gt[i]));
    }
    block_reduce<0, true>(v, sh);
    if (tid == 0) {
      S.f = E;
      S.gnorm = v[0];
    }
    __syncthreads();
    finish(S, 1.0, h, cond);
    return;
  }
  enum { A_BEGIN, A_FAIL, A_EVAL, A_STOP_OK, A_STOP_FAIL, A_STOP_CAP };
  int act;
  if (S.phase == PH_INIT) {
    double v[2] = {0.0, 0.0};  // g.g, max |g|
    for (int i = tid; i < a.nv; i += kStepThreads) {
      const double gi = a.gt[i];
      a.g[i] = gi;
      a.p[i] = -gi;
      v[0] += gi * gi;
      v[1] = nanmax(v[1], fabs(gi));
    }
    block_reduce<1, true>(v, sh);
    if (tid == 0) {
      S.f = E;
      S.f_prev = E + sqrt(v[0]) / 2.0;
      S.gnorm = v[1];
      S.delta = v[0];
      S.d0 = -v[0];
    }
    __syncthreads();  // every thread reads S.gnorm next
    act = A_BEGIN;
  } else {
    // one pass for the whole step: g1.p (the search's slope), (g1 - g).g1,
    // g1.g1, max |g1| at the trial point
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int i = tid; i < a.nv; i += kStepThreads) {
      const double gi = a.gt[i];
      v[0] += gi * a.p[i];
      v[1] += (gi - a.g[i]) * gi;
      v[2] += gi * gi;
      v[3] = nanmax(v[3], fabs(gi));
    }
    block_reduce<3, true>(v, sh);
    if (tid == 0) s_act = ls_step(S, E, v[0]);
    __syncthreads();
    const int task = s_act;
    __syncthreads();
    if (task == T_FG) {
      act = A_EVAL;
    } else if (task == T_CONV) {
      const double r = v[1] / S.delta;
      const double beta = r > 0.0 ? r : 0.0;
      // p1 = -g1 + beta p: p1.g1 = -g1.g1 + beta g1.p
      const double pg = -v[2] + beta * v[0];
      if (v[3] <= a.gtol || pg <= -0.01 * v[2]) {
        for (int i = tid; i < a.nv; i += kStepThreads) {
          a.x[i] = a.xt[i];
          a.p[i] = -a.gt[i] + beta * a.p[i];
          a.g[i] = a.gt[i];
        }
        if (tid == 0) {
          S.f_prev = S.f;
          S.f = E;
          S.gnorm = v[3];
          S.delta = v[2];
          S.d0 = pg;
          S.k += 1;
          S.restarted = 0;
        }
        act = A_BEGIN;
      } else {
        act = A_FAIL;
      }
    } else {
      act = A_FAIL;
    }
    __syncthreads();
  }
  // at most: fail -> begin (restarted) -> fail -> stop
  for (int guard = 0; guard < 4; ++guard) {
    if (act == A_FAIL) {
      int ne = 0;
      for (int i = tid; i < a.nv; i += kStepThreads) ne |= (a.p[i] != -a.g[i]);
      const int alleq = __syncthreads_or(ne) == 0;
      if (S.restarted || alleq) {
        act = A_STOP_FAIL;
      } else {
        for (int i = tid; i < a.nv; i += kStepThreads) a.p[i] = -a.g[i];
        __syncthreads();
        if (tid == 0) {
          S.restarted = 1;
          S.d0 = -S.delta;  // p = -g
        }
        act = A_BEGIN;
      }
      __syncthreads();
    }
    if (act == A_BEGIN) {
      if (!(S.gnorm > a.gtol) || S.k >= a.maxiter) {
        act = A_STOP_OK;
      } else {
        if (tid == 0) {
          const double d0 = S.d0;
          double alpha1 = 1.0;
          if (d0 != 0.0) {
            const double v = 1.01 * 2 * (S.f - S.f_prev) / d0;
            alpha1 = v < 1.0 ? v : 1.0;  // min(1, v) with Python's argument order
            if (alpha1 < 0.0) alpha1 = 1.0;
          }
          s_act = ls_start(S, alpha1, S.f, d0);
        }
        __syncthreads();
        act = s_act == T_FG ? A_EVAL : A_FAIL;
        __syncthreads();
      }
    }
    if (act != A_FAIL && act != A_BEGIN) break;
  }
  if (act == A_EVAL && S.nev >= S.maxev) act = A_STOP_CAP;
  if (act == A_EVAL) {
    const double stp = S.stp;
    for (int i = tid; i < a.nv; i += kStepThreads) a.xt[i] = a.x[i] + stp * a.p[i];
    __syncthreads();
    prep_point(a, a.xt);
    if (tid == 0) S.phase = PH_LS;
    return;
  }
  __syncthreads();
  const double success = act == A_STOP_CAP ? -1.0 : (act == A_STOP_OK && S.gnorm <= a.gtol ? 1.0 : 0.0);
  finish(S, success, h, cond);
}

// the occupations at the result (one CTA), then C^J, C^K (grid)
__global__ void __launch_bounds__(kStepThreads, kMinBlocks) occ_final_kernel(const OccState* __restrict__ st) {
  const OccArgs& a = st->a;
  if (!a.n_out && !a.cj_out) return;
  prep_point(a, a.x);
  if (a.n_out)
    for (int i = threadIdx.x; i < a.P; i += kStepThreads) a.n_out[i] = a.n[i];
}

// CJCKD8 (pnof.py:350-422) at the result's occupations, diagonals included:
// C^J = 2 n n^T, C^K = n n^T, plus on S x W, W x S, W x W the fi fi^T and
// +-nd12 nd12^T - nd nd^T terms; inside each pair block C^J = 0 and
// C^K = sqrt(n_s n_w) (strong-weak), -sqrt(n_w n_w') (weak-weak).  The
// elementwise order of the numpy expressions, without contraction.
__global__ void __launch_bounds__(kStepThreads, kMinBlocks) occ_cjck_kernel(const OccState* __restrict__ st) {
  const OccArgs& a = st->a;
  if (!a.cj_out || !a.ck_out) return;
  const int P = a.P, nb = a.no1 + a.ndoc, na = nb;
  const long long total = (long long)P * P;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t / P), j = (int)(t - (long long)i * P);
    const double ni = a.n[i], nj = a.n[j];
    double cj = __dmul_rn(2.0, __dmul_rn(ni, nj));
    double ck = __dmul_rn(ni, nj);
    const bool Si = i >= a.no1 && i < nb, Sj = j >= a.no1 && j < nb, Wi = i >= na, Wj = j >= na;
    if ((Si && Wj) || (Wi && Sj) || (Wi && Wj)) ck = __dadd_rn(ck, __dmul_rn(a.fi[i], a.fi[j]));
    if ((Si && Wj) || (Wi && Sj))
      ck = __dadd_rn(ck, __dsub_rn(__dmul_rn(a.nd12[i], a.nd12[j]), __dmul_rn(a.nd[i], a.nd[j])));
    if (Wi && Wj) ck = __dadd_rn(ck, __dsub_rn(-__dmul_rn(a.nd12[i], a.nd12[j]), __dmul_rn(a.nd[i], a.nd[j])));
    const int pi = a.pair_of[i], pj = a.pair_of[j];
    if (pi >= 0 && pi == pj) {
      const bool si = i == a.no1 + pi, sj = j == a.no1 + pj;
      if (!(si && sj)) {
        cj = 0.0;
        if (si || sj)
          ck = sqrt(__dmul_rn(a.n[si ? i : j], a.n[si ? j : i]));
        else
          ck = -sqrt(__dmul_rn(ni, nj));
      }
    }
    a.cj_out[t] = cj;
    a.ck_out[t] = ck;
  }
}

// ---- workspace and graphs
template <class Cv>
void occ_layout(Cv& c, int P, int ndoc, int ncwo, OccState** state, OccArgs& a) {
  const int nv = ndoc * ncwo, nbc = (P + kBch - 1) / kBch;
  *state = c.template take<OccState>(1);
  a.x = c.template take<double>(nv);
  a.g = c.template take<double>(nv);
  a.p = c.template take<double>(nv);
  a.pn = c.template take<double>(nv);
  a.xt = c.template take<double>(nv);
  a.gt = c.template take<double>(nv);
  a.nw = c.template take<double>(nv);
  a.n = c.template take<double>(P);
  a.nd = c.template take<double>(P);
  a.nd12 = c.template take<double>(P);
  a.fi = c.template take<double>(P);
  a.fid = c.template take<double>(P);
  a.sq = c.template take<double>(P);
  a.rsq = c.template take<double>(P);
  a.e = c.template take<double>(P);
  a.en = c.template take<double>(P);
  a.ns = c.template take<double>(ndoc);
  a.F = c.template take<double>(ndoc);
  a.dF = c.template take<double>(ndoc);
  a.part = c.template take<double>((size_t)5 * P * nbc);
  a.row = c.template take<double>((size_t)5 * P);
  a.pair_of = c.template take<int>(P);
  a.cls = c.template take<int>(P);
  a.grp = c.template take<unsigned int>((P + 31) / 32);
  a.nv = nv;
  a.nbc = nbc;
}

struct OccGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t init = nullptr;
  // host-driven form: kChunk evaluations as an ordinary graph
  cudaGraph_t chunk_graph = nullptr;
  cudaGraphExec_t chunk_exec = nullptr;
};

constexpr int kChunk = 8;  // evaluations per replay of the host-driven form

std::mutex g_mu;
// (context id, workspace, nbf5) -> graph; a context re-created after
// cudaDeviceReset has a new id, so a stale graph is never reused
std::map<std::tuple<unsigned long long, const void*, int>, OccGraph> g_graphs;

int build_graph(OccState* st, int P, OccGraph& og) {
  cudaGraph_t g = nullptr;
  GB_TRY(gb::cuda_status(cudaGraphCreate(&g, 0), "occ graph create"));
  auto fail = [&](cudaError_t e, const char* where) {
    cudaGraphDestroy(g);
    return gb::cuda_status(e, where);
  };
  OccArgs dummy{};
  void* ip[] = {&st, &dummy};
  cudaKernelNodeParams kp{};
  kp.func = (void*)occ_init_kernel;
  kp.gridDim = dim3(1);
  kp.blockDim = dim3(kStepThreads);
  kp.kernelParams = ip;
  cudaGraphNode_t init = nullptr, wn = nullptr, n4 = nullptr, n5 = nullptr;
  cudaError_t e = cudaGraphAddKernelNode(&init, g, nullptr, 0, &kp);
  if (e != cudaSuccess) return fail(e, "occ graph: init node");
  cudaGraphConditionalHandle h;
  e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return fail(e, "occ graph: conditional handle");
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  e = cudaGraphAddNode(&wn, g, &init, nullptr, 1, &cp);
  if (e != cudaSuccess) return fail(e, "occ graph: while node");
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  void* sp[] = {&st};
  int cond = 1;
  void* hp[] = {&st, &h, &cond};
  cudaKernelNodeParams r{};
  r.func = (void*)occ_rows_kernel;
  // one warp per item (the kernel strides over items beyond kRowCtas)
  const int items = ((P + 31) / 32) * ((P + kBch - 1) / kBch);
  r.gridDim = dim3(items < kRowCtas ? items : kRowCtas);
  r.blockDim = dim3(32);
  r.kernelParams = sp;
  cudaKernelNodeParams sk{};
  sk.func = (void*)occ_step_kernel;
  sk.gridDim = dim3(1);
  sk.blockDim = dim3(kStepThreads);
  sk.kernelParams = hp;
  cudaGraphNode_t prev = nullptr;
  for (int u = 0; u < kUnroll; ++u) {
    cudaGraphNode_t n1 = nullptr, n2 = nullptr;
    e = cudaGraphAddKernelNode(&n1, body, prev ? &prev : nullptr, prev ? 1 : 0, &r);
    if (e != cudaSuccess) return fail(e, "occ graph: rows node");
    e = cudaGraphAddKernelNode(&n2, body, &n1, 1, &sk);
    if (e != cudaSuccess) return fail(e, "occ graph: step node");
    prev = n2;
  }
  cudaKernelNodeParams fk{};
  fk.func = (void*)occ_final_kernel;
  fk.gridDim = dim3(1);
  fk.blockDim = dim3(kStepThreads);
  fk.kernelParams = sp;
  e = cudaGraphAddKernelNode(&n4, g, &wn, 1, &fk);
  if (e != cudaSuccess) return fail(e, "occ graph: final node");
  cudaKernelNodeParams ck{};
  ck.func = (void*)occ_cjck_kernel;
  ck.gridDim = dim3(kCjckCtas);
  ck.blockDim = dim3(kStepThreads);
  ck.kernelParams = sp;
  e = cudaGraphAddKernelNode(&n5, g, &n4, 1, &ck);
  if (e != cudaSuccess) return fail(e, "occ graph: cjck node");
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, g, 0);
  if (e != cudaSuccess) return fail(e, "occ graph: instantiate");
  og.graph = g;
  og.exec = exec;
  og.init = init;
  return GB_OK;
}

// kChunk rounds of rows -> step as an ordinary graph (no conditional node:
// the kernels return at once after the minimiser stopped)
int build_chunk_graph(OccState* st, int P, OccGraph& og) {
  cudaGraph_t g = nullptr;
  GB_TRY(gb::cuda_status(cudaGraphCreate(&g, 0), "occ chunk graph create"));
  auto fail = [&](cudaError_t e, const char* where) {
    cudaGraphDestroy(g);
    return gb::cuda_status(e, where);
  };
  void* sp[] = {&st};
  cudaGraphConditionalHandle h = 0;
  int cond = 0;
  void* hp[] = {&st, &h, &cond};
  cudaKernelNodeParams r{};
  r.func = (void*)occ_rows_kernel;
  const int items = ((P + 31) / 32) * ((P + kBch - 1) / kBch);
  r.gridDim = dim3(items < kRowCtas ? items : kRowCtas);
  r.blockDim = dim3(32);
  r.kernelParams = sp;
  cudaKernelNodeParams sk{};
  sk.func = (void*)occ_step_kernel;
  sk.gridDim = dim3(1);
  sk.blockDim = dim3(kStepThreads);
  sk.kernelParams = hp;
  cudaGraphNode_t prev = nullptr;
  for (int u = 0; u < kChunk; ++u) {
    cudaGraphNode_t n1 = nullptr, n2 = nullptr;
    cudaError_t e = cudaGraphAddKernelNode(&n1, g, prev ? &prev : nullptr, prev ? 1 : 0, &r);
    if (e != cudaSuccess) return fail(e, "occ chunk graph: rows node");
    e = cudaGraphAddKernelNode(&n2, g, &n1, 1, &sk);
    if (e != cudaSuccess) return fail(e, "occ chunk graph: step node");
    prev = n2;
  }
  cudaGraphExec_t exec = nullptr;
  cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
  if (e != cudaSuccess) return fail(e, "occ chunk graph: instantiate");
  og.chunk_graph = g;
  og.chunk_exec = exec;
  return GB_OK;
}

// The host-driven minimisation: init, then replays of the chunk graph until
// the phase copied back reads done (at most the evaluation cap's worth of
// replays), then the occupations and C^J, C^K.  The phase comes back through
// a stream-ordered copy to pageable memory (it returns once the replay has
// run), so nothing synchronises more than `s`.
int run_host_driven(OccState* st, const OccArgs& a, const OccGraph& og, cudaStream_t s, const char* name) {
  occ_init_kernel<<<1, kStepThreads, 0, s>>>(st, a);
  GB_CHECK_LAUNCH(name);
  const long long maxev = 1 + 200LL * (a.maxiter + 1);
  const long long max_replays = maxev / kChunk + 2;
  int phase = PH_INIT;
  for (long long r = 0; r < max_replays && phase != PH_DONE; ++r) {
    GB_TRY(gb::cuda_status(cudaGraphLaunch(og.chunk_exec, s), name));
    GB_TRY(gb::cuda_status(cudaMemcpyAsync(&phase, reinterpret_cast<const char*>(st) + offsetof(OccState, phase),
                                           sizeof(int), cudaMemcpyDeviceToHost, s),
                           name));
    GB_TRY(gb::cuda_status(cudaStreamSynchronize(s), name));
  }
  GB_REQUIRE(phase == PH_DONE, GB_ERR_TIMEOUT, "%s: the minimiser did not stop within the evaluation cap", name);
  occ_final_kernel<<<1, kStepThreads, 0, s>>>(st);
  GB_CHECK_LAUNCH(name);
  occ_cjck_kernel<<<kCjckCtas, kStepThreads, 0, s>>>(st);
  GB_CHECK_LAUNCH(name);
  return GB_OK;
}

int occ_run(const double* gamma0, const double* J, const double* K, const double* H, int nbf5, int no1, int ndoc,
            int ncwo, double gtol, int maxiter, int mode, double* gamma_out, double* grad_out, double* result,
            double* n_out, double* cj_out, double* ck_out, void* ws, size_t ws_bytes, void* stream,
            const char* name, bool host_driven = false) {
  gb::clear_error();
  GB_REQUIRE(gamma0 && J && K && H && result && ws, GB_ERR_INVALID_ARG, "%s: null pointer", name);
  GB_REQUIRE(mode == MODE_EVAL || gamma_out, GB_ERR_INVALID_ARG, "%s: null gamma_out", name);
  GB_REQUIRE((cj_out == nullptr) == (ck_out == nullptr), GB_ERR_INVALID_ARG, "%s: give both cj12 and ck12 or neither",
             name);
  GB_REQUIRE(no1 >= 0 && ndoc >= 1 && ncwo >= 1 && (long long)no1 + (long long)ndoc * (1 + ncwo) <= nbf5,
             GB_ERR_BAD_SHAPE, "%s: need no1 + ndoc (1 + ncwo) <= nbf5 (%d, %d, %d, %d)", name, no1, ndoc, ncwo,
             nbf5);
  GB_REQUIRE(maxiter >= 0 && gtol >= 0.0, GB_ERR_INVALID_ARG, "%s: need maxiter >= 0 and gtol >= 0", name);
  GB_REQUIRE(reinterpret_cast<uintptr_t>(ws) % 256 == 0, GB_ERR_INVALID_ARG, "%s: workspace not 256-byte aligned",
             name);
  gb::SizeCarve sc;
  OccState* dummy;
  OccArgs a{};
  occ_layout(sc, nbf5, ndoc, ncwo, &dummy, a);
  GB_REQUIRE(ws_bytes >= sc.used, GB_ERR_WORKSPACE, "%s: workspace of %zu bytes, need %zu", name, ws_bytes, sc.used);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  GB_TRY(gb::cuda_status(cudaStreamIsCapturing(s, &cs), name));
  GB_REQUIRE(cs == cudaStreamCaptureStatusNone, GB_ERR_UNSUPPORTED, "%s: not capturable (runs its own graph)", name);
  gb::Carve c(ws, ws_bytes);
  OccState* st = nullptr;
  occ_layout(c, nbf5, ndoc, ncwo, &st, a);
  a.J = J;
  a.K = K;
  a.H = H;
  a.gamma0 = gamma0;
  a.gamma_out = gamma_out ? gamma_out : a.x;
  a.grad_out = grad_out;
  a.res = result;
  a.n_out = n_out;
  a.cj_out = cj_out;
  a.ck_out = ck_out;
  a.P = nbf5;
  a.no1 = no1;
  a.ndoc = ndoc;
  a.ncwo = ncwo;
  a.maxiter = maxiter;
  a.mode = mode;
  a.gtol = gtol;
  std::unique_lock<std::mutex> lk(g_mu);
  const auto key = std::make_tuple(gb::current_context_id(), (const void*)ws, nbf5);
  auto it = g_graphs.find(key);
  if (it == g_graphs.end()) {
    OccGraph og;
    GB_TRY(build_graph(st, nbf5, og));
    it = g_graphs.emplace(key, og).first;
  }
  if (host_driven) {
    if (!it->second.chunk_exec) GB_TRY(build_chunk_graph(st, nbf5, it->second));
    // the replay loop runs without the cache lock (other workspaces' calls
    // proceed meanwhile); this workspace's entry stays until gb_occ_release,
    // which must not overlap a call on the same workspace
    const OccGraph og = it->second;
    lk.unlock();
    const int pi = gb::prof_begin(name, s);
    const int rc = run_host_driven(st, a, og, s, name);
    gb::prof_end(pi, s);
    return rc;
  }
  void* ip[] = {&st, &a};
  cudaKernelNodeParams kp{};
  kp.func = (void*)occ_init_kernel;
  kp.gridDim = dim3(1);
  kp.blockDim = dim3(kStepThreads);
  kp.kernelParams = ip;
  GB_TRY(gb::cuda_status(cudaGraphExecKernelNodeSetParams(it->second.exec, it->second.init, &kp), name));
  const int pi = gb::prof_begin(name, s);
  const cudaError_t e = cudaGraphLaunch(it->second.exec, s);
  gb::prof_end(pi, s);
  return gb::cuda_status(e, name);
}

}  // namespace

extern "C" size_t gb_occ_workspace_bytes(int nbf5, int ndoc, int ncwo) {
  if (nbf5 < 1 || ndoc < 1 || ncwo < 1) return 0;
  gb::SizeCarve sc;
  OccState* st;
  OccArgs a{};
  occ_layout(sc, nbf5, ndoc, ncwo, &st, a);
  return sc.used;
}

extern "C" int gb_occ_minimize_dev(const double* gamma0, const double* J_MO, const double* K_MO,
                                   const double* H_core, int nbf5, int no1, int ndoc, int ncwo, double gtol,
                                   int maxiter, double* gamma_out, double* result, double* n_out, double* cj12_out,
                                   double* ck12_out, void* ws, size_t ws_bytes, void* stream) {
  return occ_run(gamma0, J_MO, K_MO, H_core, nbf5, no1, ndoc, ncwo, gtol, maxiter, MODE_MIN, gamma_out, nullptr,
                 result, n_out, cj12_out, ck12_out, ws, ws_bytes, stream, "gb_occ_minimize_dev");
}

extern "C" int gb_occ_minimize_dev_sync(const double* gamma0, const double* J_MO, const double* K_MO,
                                        const double* H_core, int nbf5, int no1, int ndoc, int ncwo, double gtol,
                                        int maxiter, double* gamma_out, double* result, double* n_out,
                                        double* cj12_out, double* ck12_out, void* ws, size_t ws_bytes, void* stream) {
  return occ_run(gamma0, J_MO, K_MO, H_core, nbf5, no1, ndoc, ncwo, gtol, maxiter, MODE_MIN, gamma_out, nullptr,
                 result, n_out, cj12_out, ck12_out, ws, ws_bytes, stream, "gb_occ_minimize_dev_sync", true);
}

extern "C" int gb_occ_energy_grad_dev(const double* gamma, const double* J_MO, const double* K_MO,
                                      const double* H_core, int nbf5, int no1, int ndoc, int ncwo, double* result,
                                      double* grad, void* ws, size_t ws_bytes, void* stream) {
  return occ_run(gamma, J_MO, K_MO, H_core, nbf5, no1, ndoc, ncwo, 0.0, 0, MODE_EVAL, nullptr, grad, result,
                 nullptr, nullptr, nullptr, ws, ws_bytes, stream, "gb_occ_energy_grad_dev");
}

extern "C" int gb_occ_release(const void* ws) {
  gb::clear_error();
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto it = g_graphs.begin(); it != g_graphs.end();) {
    if (std::get<1>(it->first) == ws) {
      cudaGraphExecDestroy(it->second.exec);
      cudaGraphDestroy(it->second.graph);
      if (it->second.chunk_exec) cudaGraphExecDestroy(it->second.chunk_exec);
      if (it->second.chunk_graph) cudaGraphDestroy(it->second.chunk_graph);
      it = g_graphs.erase(it);
    } else {
      ++it;
    }
  }
  return GB_OK;
}
