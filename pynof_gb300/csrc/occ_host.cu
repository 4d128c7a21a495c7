// Occupation energy and gradient on the host (the occupation optimiser's
// inner function).  scipy's CG evaluates them thousands of times per
// occupation step at fixed J_MO, K_MO, H_core, on nbf5-sized data: the work is
// O(nbf5^2) and small, so a compiled loop replaces numpy's many small array
// operations.
//
// Follows pnof.py:
//  - occupations from the softmax parameterisation (ocupacion_softmax,
//    pnof.py:770-809): one softmax per pair over the strong orbital (logit 0)
//    and its ncwo weak partners; the strong occupation is written at index i
//    of pair i, as the reference does;
//  - the GNOF coefficients C^J, C^K (CJCKD8, pnof.py:350-422) and the
//    closed-shell energy (calce, pnof.py:905-929, diagonals of C^J, C^K zero);
//  - the gradient (calcoccg, pnof.py:1004-1033, with der_CJCKD8,
//    pnof.py:425-525): g = dn^T (2 H + diag J) + 2 sum_ij Dcj_ijk J_ji
//    - 2 sum_ij Dck_ijk K_ji, where Dc_ijk differentiates the (i, j) entry in
//    its first index.  Every such derivative is (d/dn_i of the entry) dn_ik,
//    except the dynamic terms' nd_i = n_i F(n_s) (pnof.py:364-372), which
//    also move with the pair's strong n_s.  So g = dn^T e, with e collected
//    here per orbital (and per nd_i, then chained to n_i and n_s), with the
//    1e-15 floors of the reference's denominators.
// The energy is summed with compensation (its FP64 sums carry their rounding
// errors), the occupation-space energy sums being kept in compensated FP64.
// Closed shell without singly occupied orbitals (MSpin = 0, nsoc = 0).
#include <cmath>
#include <vector>

#include "gb_common.cuh"

namespace {

constexpr double kHCut = 0.02 * 1.4142135623730951;  // H_CUT = 0.02 sqrt(2)

// Neumaier's compensated summation (A. Neumaier, ZAMM 54 (1974) 39-51): the
// rounding error of every addition is accumulated separately in c.
struct CompSum {
  double s = 0.0, c = 0.0;
  void add(double x) {
    const double t = s + x;
    c += std::fabs(s) >= std::fabs(x) ? (s - t) + x : (x - t) + s;
    s = t;
  }
  void add(const CompSum& o) {
    add(o.s);
    add(o.c);
  }
  double value() const { return s + c; }
};

struct OccLayout {
  int P, no1, ndoc, ncwo, nb;
  int strong(int p) const { return no1 + p; }
  int weak(int p, int j) const { return no1 + ndoc + (ndoc - p - 1) + ndoc * j; }
  int gam(int p, int j) const { return (ndoc - p - 1) + ndoc * j; }
};

}  // namespace

extern "C" int gb_occ_energy_grad_f64(const double* gamma, const double* J, const double* K, const double* H,
                                      int nbf5, int no1, int ndoc, int ncwo, double* energy, double* grad) {
  gb::clear_error();
  GB_REQUIRE(gamma && J && K && H && energy, GB_ERR_INVALID_ARG, "gb_occ_energy_grad_f64: null pointer");
  GB_REQUIRE(no1 >= 0 && ndoc >= 1 && ncwo >= 1 && (long long)no1 + (long long)ndoc * (1 + ncwo) <= nbf5,
             GB_ERR_BAD_SHAPE, "gb_occ_energy_grad_f64: need no1 + ndoc (1 + ncwo) <= nbf5 (%d, %d, %d, %d)", no1,
             ndoc, ncwo, nbf5);
  const OccLayout L{nbf5, no1, ndoc, ncwo, no1 + ndoc};
  const int P = nbf5;
  std::vector<double> n(P, 0.0), nd(P, 0.0), nd12(P, 0.0), fi(P, 0.0), fid(P, 0.0), e(P, 0.0), end_(P, 0.0);
  std::vector<double> ns(ndoc), nw((size_t)ndoc * ncwo), F(ndoc), dF(ndoc);
  std::vector<int> pair_of(P, -1), cls(P, 0);

  // softmax occupations
  for (int p = 0; p < ndoc; ++p) {
    double top = -INFINITY, den = 1.0;
    for (int j = 0; j < ncwo; ++j) top = std::fmax(top, gamma[L.gam(p, j)]);
    if (top >= 700.0) {
      // logits past exp's range: the same softmax shifted by the largest one
      den = std::exp(-top);
      for (int j = 0; j < ncwo; ++j) den += std::exp(gamma[L.gam(p, j)] - top);
      ns[p] = std::exp(-top) / den;
      for (int j = 0; j < ncwo; ++j) nw[(size_t)p * ncwo + j] = std::exp(gamma[L.gam(p, j)] - top) / den;
    } else {
      for (int j = 0; j < ncwo; ++j) den += std::exp(std::fmin(gamma[L.gam(p, j)], 700.0));
      ns[p] = 1.0 / den;
      for (int j = 0; j < ncwo; ++j) nw[(size_t)p * ncwo + j] = std::exp(std::fmin(gamma[L.gam(p, j)], 700.0)) / den;
    }
    n[p] = ns[p];
    for (int j = 0; j < ncwo; ++j) n[L.weak(p, j)] = nw[(size_t)p * ncwo + j];
  }
  for (int p = 0; p < ndoc; ++p) {
    pair_of[L.strong(p)] = p;
    for (int j = 0; j < ncwo; ++j) pair_of[L.weak(p, j)] = p;
  }
  for (int i = 0; i < P; ++i) cls[i] = i < no1 ? 0 : (i < L.nb ? 1 : 2);  // 1: strong set S, 2: weak set W
  for (int p = 0; p < ndoc; ++p) {
    const int s = L.strong(p);
    const double coc = (1.0 - n[s]) / kHCut;
    F[p] = std::exp(-coc * coc);
    dF[p] = 2.0 * coc / kHCut;  // (1/F) dF/dn_s
    nd[s] = n[s] * F[p];
    for (int j = 0; j < ncwo; ++j) nd[L.weak(p, j)] = n[L.weak(p, j)] * F[p];
  }
  for (int i = 0; i < P; ++i) {
    nd12[i] = std::sqrt(nd[i]);
    fi[i] = std::sqrt(std::fmax(n[i] * (1.0 - n[i]), 0.0));
    fid[i] = i < no1 ? 0.0 : (1.0 - 2.0 * n[i]) / (2.0 * std::fmax(fi[i], 1e-15));
  }

  // energy and dE/dn (e), dE/dnd (end_); pairs (a, b), a != b, of different pairs
  CompSum E;
  for (int i = 0; i < P; ++i) {
    E.add(n[i] * (2.0 * H[i] + J[(size_t)i * P + i]));
    e[i] = 2.0 * H[i] + J[(size_t)i * P + i];
  }
  for (int a = 0; a < P; ++a) {
    const int pa = pair_of[a];
    double ea = 0.0, enda = 0.0;
    CompSum Ea;
    for (int b = 0; b < P; ++b) {
      if (b == a || (pa >= 0 && pair_of[b] == pa)) continue;
      const double Jba = J[(size_t)b * P + a], Kba = K[(size_t)b * P + a];
      Ea.add(2.0 * n[a] * n[b] * Jba);
      ea += 4.0 * n[b] * Jba;
      double ck = n[a] * n[b], dck = n[b];
      const bool chi = (cls[a] == 1 && cls[b] == 2) || (cls[a] == 2 && cls[b] >= 1);
      if (chi) {
        const double sigma = (cls[a] == 2 && cls[b] == 2) ? -1.0 : 1.0;
        ck += fi[a] * fi[b] + sigma * nd12[a] * nd12[b] - nd[a] * nd[b];
        dck += fid[a] * fi[b];
        enda -= 2.0 * (sigma * nd12[b] / (2.0 * std::fmax(nd12[a], 1e-15)) - nd[b]) * Kba;
      }
      Ea.add(-ck * Kba);
      ea -= 2.0 * dck * Kba;
    }
    E.add(Ea);
    e[a] += ea;
    end_[a] += enda;
  }
  // pairs inside one pair block: C^J = 0; C^K = sqrt(n_s n_w) (strong-weak),
  // -sqrt(n_w n_w') (weak-weak)
  for (int p = 0; p < ndoc; ++p) {
    const int s = L.strong(p);
    const double rs = std::sqrt(std::fmax(n[s], 1e-15));
    for (int j = 0; j < ncwo; ++j) {
      const int w = L.weak(p, j);
      const double Kws = K[(size_t)w * P + s], Ksw = K[(size_t)s * P + w];
      const double rw = std::sqrt(std::fmax(n[w], 1e-15));
      E.add(-std::sqrt(n[s] * n[w]) * (Kws + Ksw));
      e[s] -= std::sqrt(n[w]) / rs * Kws;
      e[w] -= std::sqrt(n[s]) / rw * Ksw;
      for (int j2 = 0; j2 < ncwo; ++j2) {
        if (j2 == j) continue;
        const int w2 = L.weak(p, j2);
        const double Kw2w = K[(size_t)w2 * P + w];
        E.add(std::sqrt(n[w] * n[w2]) * Kw2w);
        e[w] += std::sqrt(n[w2]) / rw * Kw2w;
      }
    }
  }
  *energy = E.value();
  if (!grad) return GB_OK;
  // nd_s = n_s F(n_s), nd_w = n_w F(n_s)
  for (int p = 0; p < ndoc; ++p) {
    const int s = L.strong(p);
    e[s] += end_[s] * F[p] * (1.0 + n[s] * dF[p]);
    for (int j = 0; j < ncwo; ++j) {
      const int w = L.weak(p, j);
      e[w] += end_[w] * F[p];
      e[s] += end_[w] * n[w] * F[p] * dF[p];
    }
  }
  // gradient: dn^T e, dn block-sparse (row p holds the strong occupation)
  for (int p = 0; p < ndoc; ++p) {
    double wsum = 0.0;
    for (int i = 0; i < ncwo; ++i) wsum += nw[(size_t)p * ncwo + i] * e[L.weak(p, i)];
    for (int j = 0; j < ncwo; ++j) {
      const double w = nw[(size_t)p * ncwo + j];
      grad[L.gam(p, j)] = -ns[p] * w * e[p] + w * e[L.weak(p, j)] - w * wsum;
    }
  }
  return GB_OK;
}

// calce (pnof.py:905-929) for given coefficients: E = 2 sum_i n_i H_i
// + sum_{i < nbeta} n_i J_ii + sum_{i >= nalpha} n_i J_ii
// + sum_ij cj12_ij J_ji - sum_ij ck12_ij K_ji, with the compensated sum
// (the caller zeroes the coefficients' diagonals, as the reference does).
extern "C" int gb_calce_f64(const double* n, const double* cj12, const double* ck12, const double* J,
                            const double* K, const double* H, int nbf5, int nbeta, int nalpha, double* energy) {
  gb::clear_error();
  GB_REQUIRE(n && cj12 && ck12 && J && K && H && energy, GB_ERR_INVALID_ARG, "gb_calce_f64: null pointer");
  GB_REQUIRE(nbf5 >= 1 && 0 <= nbeta && nbeta <= nalpha && nalpha <= nbf5, GB_ERR_BAD_SHAPE,
             "gb_calce_f64: need 0 <= nbeta <= nalpha <= nbf5 (%d, %d, %d)", nbeta, nalpha, nbf5);
  const int P = nbf5;
  CompSum E;
  for (int i = 0; i < P; ++i) E.add(2.0 * n[i] * H[i]);
  for (int i = 0; i < nbeta; ++i) E.add(n[i] * J[(size_t)i * P + i]);
  for (int i = nalpha; i < P; ++i) E.add(n[i] * J[(size_t)i * P + i]);
  for (int a = 0; a < P; ++a)
    for (int b = 0; b < P; ++b) {
      E.add(cj12[(size_t)a * P + b] * J[(size_t)b * P + a]);
      E.add(-(ck12[(size_t)a * P + b] * K[(size_t)b * P + a]));
    }
  *energy = E.value();
  return GB_OK;
}
