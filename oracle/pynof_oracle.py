"""CPU oracle for the RI / full-ERI JK and MO-integral path of PyNOF.

TEST INFRASTRUCTURE ONLY.  This module is the oracle of the parity tests, the
smoke check and the CPU-baseline leg of the benchmark, which import it.  Nothing in
the ``pynof_gb300`` package imports it, and no product code path runs through
it.

It restates, in plain numpy FP64, the algorithms of PyNOF 1.4 (``src/pynof``)
for the functions the CUDA path replaces.  Each function names the reference
lines it follows.  Parity of this restatement is pinned against golden vectors
produced by the reference's own functions (``tests/golden/make_golden.py``
imports PyNOF with stub psi4/numba modules and records inputs and outputs).

Array conventions (identical to the reference): ``C`` (N, N) with MO p in
column p; ``b`` (N, N, Q) with Q fastest; ``I`` (N, N, N, N) with
``I[m, n, s, l] = (mn|sl)``; ``H`` (N, N); ``n`` (P,); ``cj12``/``ck12`` (P, P).
``p`` is any object with the ``pynof.param`` size attributes
(nbf, nbf5, nbeta, nalpha, no1, noptorb, MSpin, HighSpin, RI, ...).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg


# ----------------------------------------------------------------------------
# A1 / A2: per-orbital J_i, K_i
# ----------------------------------------------------------------------------
def jkj_ri(C, b, P):
    """J_q, K_q from the RI factor (``integrals.py:208-218`` JKj_RI).

    T[q, n, l]  = sum_m C[m, q] b[m, n, l]
    d[q, l]     = sum_n C[n, q] T[q, n, l]
    J[q, m, n]  = sum_l d[q, l] b[m, n, l]
    K[q, m, n]  = sum_l T[q, m, l] T[q, n, l]
    """
    N, _, Q = b.shape
    Cp = C[:, :P]
    T = (Cp.T @ b.reshape(N, N * Q)).reshape(P, N, Q)
    d = np.einsum("nq,qnl->ql", Cp, T)
    J = (d @ b.reshape(N * N, Q).T).reshape(P, N, N)
    K = np.matmul(T, T.transpose(0, 2, 1))
    return J, K


def jkj_full(C, I, P):
    """J_i, K_i from the 4-index tensor (``integrals.py:197-205`` JKj_Full).

    D_i = C_i C_i^T;  J_i[m, n] = sum_sl D_i[s, l] (mn|sl);
    K_i[m, s] = sum_nl D_i[n, l] (mn|sl).
    """
    N = I.shape[0]
    Cp = C[:, :P]
    D = np.einsum("mi,ni->imn", Cp, Cp)
    J = (D.reshape(P, N * N) @ I.reshape(N * N, N * N).T).reshape(P, N, N)
    # K needs (m,s) x (n,l): permute I to [m, s, n, l]
    Iperm = I.transpose(0, 2, 1, 3).reshape(N * N, N * N)
    K = (D.reshape(P, N * N) @ Iperm.T).reshape(P, N, N)
    return J, K


# ----------------------------------------------------------------------------
# A3 / A4: MO-basis J_pq, K_pq, H_pp
# ----------------------------------------------------------------------------
def hcore_diag(C, H, P):
    """H_core[p] = C_p^T H C_p (``integrals.py:345``, ``:361``)."""
    Cp = C[:, :P]
    return np.einsum("mp,mp->p", Cp, H @ Cp)


def jkh_mo_ri(C, H, b, P):
    """(pp|qq), (pq|pq), H_pp from b (``integrals.py:348-362`` JKH_MO_RI)."""
    N, _, Q = b.shape
    Cp = C[:, :P]
    T = (Cp.T @ b.reshape(N, N * Q)).reshape(P, N, Q)          # [p, n, l]
    bpq = np.matmul(Cp.T[None, :, :], T)                        # [p, q, l]
    diag = bpq[np.arange(P), np.arange(P), :]                   # [p, l]
    J_MO = diag @ diag.T
    K_MO = np.einsum("pql,pql->pq", bpq, bpq)
    return J_MO, K_MO, hcore_diag(C, H, P)


def jkh_mo_full(C, H, I, P):
    """(ii|jj), (ij|ij), H_ii from I (``integrals.py:332-345`` JKH_MO_Full)."""
    N = I.shape[0]
    Cp = C[:, :P]
    D = np.einsum("mi,ni->imn", Cp, Cp).reshape(P, N * N)
    J, K = jkj_full(C, I, P)
    J_MO = J.reshape(P, N * N) @ D.T
    K_MO = K.reshape(P, N * N) @ D.T
    return J_MO, K_MO, hcore_diag(C, H, P)


# ----------------------------------------------------------------------------
# A5 / A6: MO integrals for the Lagrangian and computeLagrange2
# ----------------------------------------------------------------------------
def integrals_mo_ri(C, H, b, P):
    """Hmat (N, P) and b_MO (N, P, Q) (``integrals.py:701-706``)."""
    N, _, Q = b.shape
    Hmat = C.T @ H @ C[:, :P]
    Cp = C[:, :P]
    # T[q, m, l] = sum_n C[n, q] b[m, n, l] (b symmetric is NOT assumed here:
    # contract the second index explicitly); both steps are batched BLAS GEMMs,
    # as the reference's einsum(..., optimize=True) is
    T = np.matmul(Cp.T[None, :, :], b).transpose(1, 0, 2)      # [m, q, l] -> [q, m, l]
    bmo = np.matmul(C.T[None, :, :], T).transpose(1, 0, 2)      # [q, a, l] -> [a, q, l]
    return Hmat, np.ascontiguousarray(bmo)


def integrals_mo_full(C, H, I, P):
    """Hmat and I_MO[p, q, r, t] (``integrals.py:685-690``); p over N, q r t over P."""
    Hmat = C.T @ H @ C[:, :P]
    Cp = C[:, :P]
    X = np.tensordot(I, Cp, axes=([3], [0]))        # m n s t
    X = np.tensordot(X, Cp, axes=([2], [0]))        # m n t r
    X = np.tensordot(X, Cp, axes=([1], [0]))        # m t r q
    X = np.tensordot(X, C, axes=([0], [0]))         # t r q p
    return Hmat, np.ascontiguousarray(X.transpose(3, 2, 1, 0))


def _zero_diag(a):
    np.fill_diagonal(a, 0.0)


def lagrange2(n, cj12, ck12, C, H, I, b, p):
    """elag (N, N) and Hmat (N, P) (``utils.py:262-382`` computeLagrange2).

    Closed shell (MSpin == 0) only, as in the reference.  The diagonals of cj12
    and ck12 are zeroed in place (``utils.py:269-270``).
    """
    N, P = p.nbf, p.nbf5
    nb, na = p.nbeta, p.nalpha
    _zero_diag(cj12)
    _zero_diag(ck12)
    elag = np.zeros((N, N))
    if p.MSpin != 0:
        # the reference assembles nothing for open shells (utils.py:272-274, :329-331)
        Hmat = C.T @ H @ C[:, :P]
        return elag, Hmat
    if p.RI:
        Hmat, bmo = integrals_mo_ri(C, H, b, P)
        bbk = bmo[np.arange(P), np.arange(P), :]                      # [b, k] = bMO[b, b, k]
        w = np.zeros_like(bbk)
        w[:nb] += n[:nb, None] * bbk[:nb]
        w[na:P] += n[na:P, None] * bbk[na:P]
        w += cj12 @ bbk                                               # sum_q cj12[b,q] bMO[q,q,k]
        elag[:, :P] += n[None, :] * Hmat[:, :P]
        elag[:, :P] += np.matmul(bmo.transpose(1, 0, 2), w[:, :, None])[:, :, 0].T  # sum_k bMO[a,b,k] w[b,k]
        Y = ck12[:, :, None] * bmo[:P]                                # [b, q, k]
        elag[:, :P] -= bmo.reshape(N, -1) @ Y.reshape(P, -1).T
    else:
        Hmat, imo = integrals_mo_full(C, H, I, P)
        ar = np.arange(P)
        elag[:, :P] += n[None, :] * Hmat[:, :P]
        diag3 = imo[:, ar, ar, ar]                                    # [a, b] = I_MO[a,b,b,b]
        elag[:, :nb] += n[None, :nb] * diag3[:, :nb]
        elag[:, na:P] += n[None, na:P] * diag3[:, na:P]
        abqq = imo[:, :, ar, ar]                                      # [a, b, q]
        elag[:, :P] += np.einsum("bq,abq->ab", cj12, abqq)
        aqbq = np.einsum("aqbq->abq", imo)                           # [a, b, q] = I_MO[a,q,b,q]
        elag[:, :P] -= np.einsum("bq,abq->ab", ck12, aqbq)
    return elag, Hmat


# ----------------------------------------------------------------------------
# A8 / A7: generalized Fock, Lagrangian, energy
# ----------------------------------------------------------------------------
def fock_rc(J, K, n, H, cj12, ck12, p):
    """F_i (P, N, N) closed shell (``utils.py:25-55`` computeF_RC_CPU).

    Zeroes diag(cj12[ini:, ini:]) and diag(ck12[ini:, ini:]) in place.
    """
    P = p.nbf5
    ini = p.no1 if p.no1 > 1 else 0
    F = n[:, None, None] * H[None, :, :]
    F = F.copy()
    F[ini:p.nbeta] += n[ini:p.nbeta, None, None] * J[ini:p.nbeta]
    F[p.nalpha:P] += n[p.nalpha:P, None, None] * J[p.nalpha:P]
    _zero_diag(cj12[ini:, ini:])
    _zero_diag(ck12[ini:, ini:])
    N = J.shape[1]
    F += (cj12 @ J.reshape(P, N * N)).reshape(P, N, N)
    F -= (ck12 @ K.reshape(P, N * N)).reshape(P, N, N)
    return F


def fock_ro(J, K, n, H, cj12, ck12, p):
    """F_i (P, N, N) restricted open shell (``utils.py:97-169`` computeF_RO_CPU).

    Index blocks: D = [0, nbeta) and [nalpha, P) (doubly occupied and
    correlating orbitals), O = [nbeta, nalpha) (singly occupied).  Step by step
    as the reference: n_i H on D and H / 2 on O; n_i J_i on [ini, nbeta) and
    [nalpha, P); the C^J J and -C^K K couplings inside D (diagonals from ini
    on zeroed in place); the D-O terms n_i sum_{j in O} (J_j - K_j / 2); for O,
    (1/2) sum_{j in O, j != i} (J_j - K_j) plus sum_{j in D} n_j (J_j - K_j / 2).
    """
    P, nb, na = p.nbf5, p.nbeta, p.nalpha
    ini = p.no1 if p.no1 > 1 else 0
    N = J.shape[1]
    D = np.r_[0:nb, na:P]
    O = np.arange(nb, na)
    F = np.zeros((P, N, N))
    F[D] += n[D, None, None] * H[None]
    F[O] += 0.5 * H[None]
    F[ini:nb] += n[ini:nb, None, None] * J[ini:nb]
    F[na:P] += n[na:P, None, None] * J[na:P]
    _zero_diag(cj12[ini:, ini:])
    _zero_diag(ck12[ini:, ini:])
    JD = J[D].reshape(len(D), N * N)
    KD = K[D].reshape(len(D), N * N)
    F[D] += (cj12[np.ix_(D, D)] @ JD - ck12[np.ix_(D, D)] @ KD).reshape(len(D), N, N)
    if len(O):
        WO = (J[O] - 0.5 * K[O]).sum(axis=0)                       # sum_{j in O} (J_j - K_j / 2)
        F[D] += n[D, None, None] * WO[None]
        VO = (J[O] - K[O]).sum(axis=0)
        F[O] += 0.5 * VO[None] - 0.5 * (J[O] - K[O])               # j != i within O
        WD = np.tensordot(n[D], J[D] - 0.5 * K[D], axes=1)         # sum_{j in D} n_j (J_j - K_j / 2)
        F[O] += WD[None]
    return F


def lagrange(F, C, p):
    """elag from F (``utils.py:249-259`` computeLagrange)."""
    P, N, no = p.nbf5, p.nbf, p.noptorb
    G = np.einsum("imn,ni->mi", F, C[:, :P])
    elag = np.zeros((N, N))
    elag[:no, :P] = (C[:, :no].T @ G)[:no, :P]
    return elag


def e_elec(H, C, n, elag, p):
    """Electronic energy (``utils.py:385-402`` computeE_elec)."""
    P, nb, na = p.nbf5, p.nbeta, p.nalpha
    hd = hcore_diag(C, H, P)
    E = np.trace(elag[:P, :P])
    E += np.dot(n[:nb], hd[:nb])
    if not p.HighSpin:
        E += np.dot(n[nb:na], hd[nb:na])
    else:
        E += 0.5 * np.sum(hd[nb:na])
    E += np.dot(n[na:P], hd[na:P])
    return E


def lagrange_convergency(elag):
    """(sumdiff, maxdiff) of elag - elag^T (``utils.py:405-411``)."""
    d = np.abs(elag - elag.T)
    return d.sum(), d.max()


def energy1r(C, n, H, I, b, cj12, ck12, p):
    """E, elag, sumdiff, maxdiff (``utils.py:414-431`` ENERGY1r)."""
    P = p.nbf5
    if p.no1 == 0:
        elag, Hmat = lagrange2(n, cj12, ck12, C, H, I, b, p)
        E = np.trace(elag[:P, :P]) + np.dot(n[:P], np.diagonal(Hmat)[:P])
    else:
        J, K = jkj_ri(C, b, P) if p.RI else jkj_full(C, I, P)
        F = fock_rc(J, K, n, H, cj12, ck12, p) if p.MSpin == 0 else fock_ro(J, K, n, H, cj12, ck12, p)
        elag = lagrange(F, C, p)
        E = e_elec(H, C, n, elag, p)
    s, m = lagrange_convergency(elag)
    return E, elag, s, m


# ----------------------------------------------------------------------------
# A9 / A10: occupation-space energy and the orbital gradient
# ----------------------------------------------------------------------------
def calce(n, cj12, ck12, J_MO, K_MO, H_core, p):
    """E(n) closed shell (``pnof.py:905-929`` calce, MSpin == 0)."""
    P, nb, na = p.nbf5, p.nbeta, p.nalpha
    dj = np.diagonal(J_MO)
    E = 2.0 * np.dot(n, H_core) + np.dot(n[:nb], dj[:nb]) + np.dot(n[na:P], dj[na:P])
    _zero_diag(cj12)
    _zero_diag(ck12)
    E += np.sum(cj12 * J_MO.T) - np.sum(ck12 * K_MO.T)
    return E


def ocupacion_softmax(x, p):
    """Occupations n (nbf5,) from the gammas (``pnof.py:770-809``): per pair
    i, one softmax over a zero logit for the strong orbital and the ncwo weak
    ones at ll, ll + ndoc, ...; the strong occupation is stored at index i (as
    the reference does); singly occupied orbitals at 0.5 (1.0 high spin)."""
    no1, ndoc, ndns, ncwo = p.no1, p.ndoc, p.ndns, p.ncwo
    n = np.zeros(p.nbf5)
    n[no1 + ndoc: no1 + ndns] = 1.0 if getattr(p, "HighSpin", False) else 0.5
    ex = np.exp(np.asarray(x, dtype=np.float64))
    for i in range(ndoc):
        ll = no1 + ndns + (ndoc - i - 1)
        llx = ndoc - i - 1
        e = ex[llx: llx + ndoc * ncwo: ndoc]
        den = 1 + np.sum(e)
        n[i] = 1 / den
        n[ll: ll + ndoc * ncwo: ndoc] = e / den
    return n


def cjckd8(n, p):
    """GNOF coefficients C^J, C^K (``pnof.py:350-422``, CJCKD8), MSpin == 0."""
    no1, ndoc, nsoc, nb, na, ndns, ncwo = p.no1, p.ndoc, p.nsoc, p.nbeta, p.nalpha, p.ndns, p.ncwo
    h_cut = 0.02 * np.sqrt(2.0)
    n_d = np.zeros(len(n))
    for i in range(ndoc):
        idx = no1 + i
        ll = no1 + ndns + (ndoc - i - 1)
        ul = ll + ndoc * ncwo
        F = np.exp(-(((1.0 - n[idx]) / h_cut) ** 2))
        n_d[idx] = n[idx] * F
        n_d[ll:ul:ndoc] = n[ll:ul:ndoc] * F
    n_d12 = np.sqrt(n_d)
    fi = n * (1 - n)
    fi[fi <= 0] = 0
    fi = np.sqrt(fi)
    cj12 = 2 * np.outer(n, n)
    ck12 = np.outer(n, n)
    ck12[no1:nb, na:] += np.outer(fi[no1:nb], fi[na:])
    ck12[na:, no1:nb] += np.outer(fi[na:], fi[no1:nb])
    ck12[na:, na:] += np.outer(fi[na:], fi[na:])
    if nsoc > 0:
        half = np.full(nsoc, 0.5)
        ck12[no1:nb, nb:na] += 0.5 * np.outer(fi[no1:nb], half)
        ck12[nb:na, no1:nb] += 0.5 * np.outer(half, fi[no1:nb])
        ck12[nb:na, na:] += np.outer(half, fi[na:])
        ck12[na:, nb:na] += np.outer(fi[na:], half)
    if nsoc > 1:
        ck12[nb:na, nb:na] = 0.5
    ck12[no1:nb, na:] += np.outer(n_d12[no1:nb], n_d12[na:]) - np.outer(n_d[no1:nb], n_d[na:])
    ck12[na:, no1:nb] += np.outer(n_d12[na:], n_d12[no1:nb]) - np.outer(n_d[na:], n_d[no1:nb])
    ck12[na:, na:] += -np.outer(n_d12[na:], n_d12[na:]) - np.outer(n_d[na:], n_d[na:])
    for i in range(ndoc):
        idx = no1 + i
        ll = no1 + ndns + (ndoc - i - 1)
        ul = ll + ndoc * ncwo
        nw = n[ll:ul:ndoc]
        cj12[idx, ll:ul:ndoc] = 0
        cj12[ll:ul:ndoc, idx] = 0
        cj12[ll:ul:ndoc, ll:ul:ndoc] = 0
        ck12[idx, ll:ul:ndoc] = np.sqrt(n[idx] * nw)
        ck12[ll:ul:ndoc, idx] = np.sqrt(n[idx] * nw)
        ck12[ll:ul:ndoc, ll:ul:ndoc] = -np.sqrt(np.outer(nw, nw))
    return cj12, ck12


def calcocce(gamma, J_MO, K_MO, H_core, p):
    """The occupation energy E(gamma) (``pnof.py:994-1001``): softmax
    occupations, GNOF coefficients, calce."""
    n = ocupacion_softmax(gamma, p)
    cj12, ck12 = cjckd8(n, p)
    return calce(n, cj12, ck12, J_MO, K_MO, H_core, p)


def orbital_gradient(elag, p):
    """Packed 4 (elag - elag^T) over i < nbf5, j > i (``pnof.py:1114-1131``)."""
    g = 4.0 * (elag - elag.T)
    iu = np.triu_indices(p.nbf, 1)
    keep = iu[0] < p.nbf5
    return g[iu[0][keep], iu[1][keep]]


def rotate_orbital(y, C, p):
    """C expm(Y) with Y antisymmetric from packed y (``utils.py:550-565``)."""
    N = p.nbf
    Y = np.zeros((N, N))
    iu = np.triu_indices(N, 1)
    keep = iu[0] < p.nbf5
    Y[iu[0][keep], iu[1][keep]] = y
    Y -= Y.T
    return C @ scipy.linalg.expm(Y)


def metric_power(metric, alpha=-0.5, cutoff=1.0e-14):
    """psi4 Matrix::power(alpha, cutoff) as ``integrals.py:45`` calls it
    (psi4 unpinned; its published behaviour): eigenvalues below cutoff x the
    largest magnitude are dropped for negative powers, the rest raised to
    alpha.  Parity unpinned: psi4 is absent here."""
    a, V = np.linalg.eigh(metric)
    amax = max(abs(a[0]), abs(a[-1]))
    out = np.zeros_like(a)
    for i, ai in enumerate(a):
        if alpha < 0.0 and abs(ai) < cutoff * amax:
            continue
        v = ai ** alpha
        out[i] = v if np.isfinite(v) else 0.0
    return V @ np.diag(out) @ V.T


def b_mnl(mnk, metric):
    """``integrals.py:45-49``: einsum("mnk,kl->mnl", mnk, metric^(-1/2))."""
    return np.einsum("mnk,kl->mnl", mnk, metric_power(metric), optimize=True)


def density_hf(C, j0, j1):
    """sum_{j0 <= j < j1} C[:, j] C[:, j]^T (``integrals.py:493-510``,
    computeD_HF with [0, nbeta), computeDalpha_HF with [nbeta, nalpha))."""
    Cs = C[:, j0:j1]
    return Cs @ Cs.T


def jk_hf_full(D, I):
    """J = einsum("ls,mnsl->mn"), K = einsum("nl,mnsl->ms") (``integrals.py:528-543``)."""
    N = D.shape[0]
    J = (I.reshape(N * N, N * N) @ D.T.reshape(-1)).reshape(N, N)
    K = np.einsum("nl,mnsl->ms", D, I, optimize=True)
    return J, K


def mo4_full(C, I, p, q, r, t):
    """sum C[m,p] C[n,q] I[m,n,s,l] C[s,r] C[l,t] over orbital ranges
    (``integrals.py:611-623`` iajb_Full_jit, ``:651-654`` pqrt_Full_jit)."""
    Cp, Cq, Cr, Ct = (C[:, a:b] for a, b in (p, q, r, t))
    return np.einsum("mp,nq,mnsl,sr,lt->pqrt", Cp, Cq, I, Cr, Ct, optimize=True)


def erpa_mo_integrals_ri(C, H, b, P):
    """``postpnof.py:1402-1406`` (RI): h and (pq|sl) from b_pql."""
    Cp = C[:, :P]
    h = np.einsum("mi,mn,nj->ij", Cp, H, Cp, optimize=True)
    b_pql = np.einsum("mnl,mp,nq->pql", b, Cp, Cp, optimize=True)
    return h, np.einsum("pqR,slR->pqsl", b_pql, b_pql, optimize=True)


def eri_from_b(b):
    """(mn|sl) = sum_Q b[m, n, Q] b[s, l, Q] (the exact RI identity)."""
    N, _, Q = b.shape
    B = b.reshape(N * N, Q)
    return (B @ B.T).reshape(N, N, N, N)
