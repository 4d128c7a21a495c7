"""Occupation-space and orbital-rotation math of the NOF solve (host, FP64).

These are the small O(P^2 nv) / O(N^3) pieces around the device contractions:
softmax occupations, the GNOF (PNOF8) coefficients and their derivatives, the
occupation energy and gradient, the packed orbital gradient and the orbital
rotation.  They stay in FP64 on the host (the rotation exponential in
particular); every function names the reference lines it restates.

``p`` is any object with the ``pynof.param`` size attributes (no1, ndoc,
nsoc, ncwo, nbeta, nalpha, ndns, nbf, nbf5, nv, nvar, MSpin, HighSpin).
Closed shell (MSpin == 0) is the supported case, as on the device path.
"""
from __future__ import annotations

import functools

import numpy as np
import scipy.linalg

H_CUT = 0.02 * np.sqrt(2.0)


def _pairs(p):
    """(strong orbital index, weak orbital indices, gamma indices) per pair.

    The weak orbitals coupled to strong orbital i are
    no1 + ndns + (ndoc - i - 1) + j * ndoc, j < ncwo (``pnof.py:360-366``)."""
    out = []
    for i in range(p.ndoc):
        w0 = p.no1 + p.ndns + (p.ndoc - i - 1)
        weak = w0 + p.ndoc * np.arange(p.ncwo)
        g0 = p.ndoc - i - 1
        gam = g0 + p.ndoc * np.arange(p.ncwo)
        out.append((p.no1 + i, weak, gam))
    return out


@functools.lru_cache(maxsize=64)
def _pair_index(no1, ndoc, ndns, ncwo):
    i = np.arange(ndoc)
    s = no1 + i
    weak = (no1 + ndns + (ndoc - i - 1))[:, None] + ndoc * np.arange(ncwo)[None, :]
    gam = (ndoc - i - 1)[:, None] + ndoc * np.arange(ncwo)[None, :]
    block = np.concatenate([s[:, None], weak], axis=1)  # (ndoc, 1 + ncwo): strong first
    return s, weak, gam, block


def ocupacion_softmax(gamma, p):
    """Occupations n (nbf5,) and dn/dgamma (nbf5, nv) from the softmax
    parameterisation (``pnof.py:770-809``): each strong orbital and its weak
    partners share one softmax with a zero logit for the strong orbital.
    All pairs at once (their index sets are disjoint)."""
    n = np.zeros(p.nbf5)
    dn = np.zeros((p.nbf5, p.nv))
    n[p.no1 + p.ndoc: p.no1 + p.ndns] = 1.0 if p.HighSpin else 0.5
    if p.ndoc == 0:
        return n, dn
    _, weak, gam, _ = _pair_index(p.no1, p.ndoc, p.ndns, p.ncwo)
    x = np.asarray(gamma)[gam]  # (ndoc, ncwo)
    top = x.max(axis=1) if p.ncwo else np.zeros(p.ndoc)
    e = np.exp(np.minimum(x, 700.0))
    den = 1.0 + e.sum(axis=1)
    ns = 1.0 / den
    nw = e / den[:, None]
    big = top >= 700.0
    if np.any(big):
        # logits a line search pushed past exp's range: the same softmax,
        # shifted by its largest logit
        xb, tb = x[big], top[big]
        eb = np.exp(xb - tb[:, None])
        denb = np.exp(-tb) + eb.sum(axis=1)
        ns[big] = np.exp(-tb) / denb
        nw[big] = eb / denb[:, None]
    rows = np.arange(p.ndoc)
    # the reference writes the strong occupation at index i (pnof.py:793)
    n[rows] = ns
    n[weak] = nw
    dn[rows[:, None], gam] = -ns[:, None] * nw
    blk = -nw[:, :, None] * nw[:, None, :]
    ar = np.arange(p.ncwo)
    blk[:, ar, ar] += nw
    dn[weak[:, :, None], gam[:, None, :]] = blk
    return n, dn


def cjckd8(n, p):
    """GNOF coefficients C^J, C^K (nbf5, nbf5) (``pnof.py:350-422``)."""
    no1, nb, na = p.no1, p.nbeta, p.nalpha
    nd = np.zeros_like(n)
    if p.ndoc:
        s, weak, _, _ = _pair_index(p.no1, p.ndoc, p.ndns, p.ncwo)
        F = np.exp(-((1.0 - n[s]) / H_CUT) ** 2)
        nd[s] = n[s] * F
        nd[weak] = n[weak] * F[:, None]
    nd12 = np.sqrt(nd)
    fi = np.sqrt(np.clip(n * (1.0 - n), 0.0, None))
    cj = 2.0 * np.outer(n, n)
    ck = np.outer(n, n)
    S, W = slice(no1, nb), slice(na, None)
    ck[S, W] += np.outer(fi[S], fi[W])
    ck[W, S] += np.outer(fi[W], fi[S])
    ck[W, W] += np.outer(fi[W], fi[W])
    if p.MSpin == 0 and p.nsoc > 0:
        O = slice(nb, na)
        half = np.full(p.nsoc, 0.5)
        ck[S, O] += 0.5 * np.outer(fi[S], half)
        ck[O, S] += 0.5 * np.outer(half, fi[S])
        ck[O, W] += np.outer(half, fi[W])
        ck[W, O] += np.outer(fi[W], half)
    if p.MSpin == 0 and p.nsoc > 1:
        ck[nb:na, nb:na] = 0.5
    ck[S, W] += np.outer(nd12[S], nd12[W]) - np.outer(nd[S], nd[W])
    ck[W, S] += np.outer(nd12[W], nd12[S]) - np.outer(nd[W], nd[S])
    ck[W, W] += -np.outer(nd12[W], nd12[W]) - np.outer(nd[W], nd[W])
    if p.ndoc:
        s, weak, _, _ = _pair_index(p.no1, p.ndoc, p.ndns, p.ncwo)
        sc = s[:, None]
        cj[sc, weak] = 0.0
        cj[weak, sc] = 0.0
        cj[weak[:, :, None], weak[:, None, :]] = 0.0
        sw = np.sqrt(n[s][:, None] * n[weak])
        ck[sc, weak] = sw
        ck[weak, sc] = sw
        ck[weak[:, :, None], weak[:, None, :]] = -np.sqrt(n[weak][:, :, None] * n[weak][:, None, :])
    return cj, ck


def der_cjckd8(n, dn, p):
    """Derivatives of C^J, C^K w.r.t. gamma, (nbf5, nbf5, nv), taken with
    respect to the first index's occupation as the reference does
    (``pnof.py:425-525``)."""
    no1, nb, na, P = p.no1, p.nbeta, p.nalpha, p.nbf5
    nd = np.zeros_like(n)
    dnd = np.zeros_like(dn)
    for s, weak, _ in _pairs(p):
        coc = (1.0 - n[s]) / H_CUT
        F = np.exp(-coc ** 2)
        dF = 2.0 * coc / H_CUT  # (1/F) dF/dn_s
        nd[s] = n[s] * F
        nd[weak] = n[weak] * F
        dnd[s] = F * dn[s] * (1.0 + n[s] * dF)
        dnd[weak] = F * (dn[weak] + dF * np.outer(n[weak], dn[s]))
    nd12 = np.sqrt(nd)
    dnd12 = 0.5 * dnd / np.maximum(nd12, 1e-15)[:, None]
    fi = np.sqrt(np.clip(n * (1.0 - n), 0.0, None))
    dfi = np.zeros_like(dn)
    dfi[no1:] = ((1.0 - 2.0 * n[no1:]) / (2.0 * np.maximum(fi[no1:], 1e-15)))[:, None] * dn[no1:]

    Dcj = 2.0 * np.einsum("ik,j->ijk", dn, n)
    Dck = np.einsum("ik,j->ijk", dn, n)
    S, W = slice(no1, nb), slice(na, P)
    # inter-pair terms: d/dn_a of f_a f_b and of the dynamic parts, a the first index
    Dck[S, W] += np.einsum("ak,b->abk", dfi[S], fi[W])
    Dck[W, S] += np.einsum("ak,b->abk", dfi[W], fi[S])
    Dck[W, W] += np.einsum("ak,b->abk", dfi[W], fi[W])
    if p.MSpin == 0 and p.nsoc > 0:
        O = slice(nb, na)
        Dck[S, O] += 0.25 * dfi[S][:, None, :]
        Dck[W, O] += 0.5 * dfi[W][:, None, :]
    if p.MSpin == 0 and p.nsoc > 1:
        Dck[nb:na, nb:na] = 0.0
    Dck[S, W] += np.einsum("ak,b->abk", dnd12[S], nd12[W]) - np.einsum("ak,b->abk", dnd[S], nd[W])
    Dck[W, S] += np.einsum("ak,b->abk", dnd12[W], nd12[S]) - np.einsum("ak,b->abk", dnd[W], nd[S])
    Dck[W, W] += -np.einsum("ak,b->abk", dnd12[W], nd12[W]) - np.einsum("ak,b->abk", dnd[W], nd[W])
    # intra-pair terms
    for s, weak, _ in _pairs(p):
        Dcj[s, weak] = 0.0
        Dcj[weak, s] = 0.0
        Dcj[np.ix_(weak, weak)] = 0.0
        a = max(n[s], 1e-15)
        bw = np.maximum(n[weak], 1e-15)
        Dck[s, weak] = 0.5 / np.sqrt(a) * np.outer(np.sqrt(n[weak]), dn[s])
        Dck[weak, s] = 0.5 / np.sqrt(bw)[:, None] * dn[weak] * np.sqrt(n[s])
        Dck[np.ix_(weak, weak)] = -0.5 * np.einsum("ak,b->abk", dn[weak] / np.sqrt(bw)[:, None], np.sqrt(n[weak]))
    return Dcj, Dck


def calce(n, cj12, ck12, J_MO, K_MO, H_core, p):
    """Closed-shell energy E(n) (``pnof.py:905-929``).  The diagonals of cj12 /
    ck12 are zeroed in place, as in the reference.  The terms are summed with
    compensation (the library's ``gb_calce_f64``, host code): the
    occupation-space energy sums are kept in compensated FP64."""
    from . import _lib

    np.fill_diagonal(cj12, 0.0)
    np.fill_diagonal(ck12, 0.0)
    args = [np.ascontiguousarray(a, dtype=np.float64) for a in (n, cj12, ck12, J_MO, K_MO, H_core)]
    E = np.zeros(1)
    _lib.call("gb_calce_f64", *(a.ctypes.data for a in args), p.nbf5, p.nbeta, p.nalpha, E.ctypes.data)
    return float(E[0])


# ---------------------------------------------------------------------------
# Occupation gradient by contraction.  calcoccg above materialises
# dC^J/dgamma and dC^K/dgamma as (nbf5, nbf5, nv) tensors and contracts them
# with J_MO, K_MO; scipy's CG calls it thousands of times per occoptr, so the
# O(nbf5^2 nv) tensors dominate a served solve.  Every term of der_cjckd8 is an
# outer product u[a, k] v[b] on a block of (a, b), so its contraction with a
# matrix Y is u[A]^T (Y[A, B] v[B]): O(nbf5^2 + nbf5 nv).  The intra-pair
# blocks, which der_cjckd8 overwrites, are corrected pair by pair on small
# (1 + ncwo)^2 blocks.  Closed shell without singly occupied orbitals (the
# served and benchmarked case); other structures use calcoccg.
# ---------------------------------------------------------------------------
def _fast_ok(p):
    return p.MSpin == 0 and p.nsoc == 0 and p.ncwo >= 1 and p.ndoc >= 1


def calcoccg_fast(gamma, J_MO, K_MO, H_core, p):
    """dE/dgamma equal to :func:`calcoccg` (same terms, contracted without
    the (nbf5, nbf5, nv) derivative tensors)."""
    if not _fast_ok(p):
        return calcoccg(gamma, J_MO, K_MO, H_core, p)
    P, no1, nb, na = p.nbf5, p.no1, p.nbeta, p.nalpha
    n, dn = ocupacion_softmax(gamma, p)
    s_idx, weak, gam, block = _pair_index(p.no1, p.ndoc, p.ndns, p.ncwo)
    # occupation-derived vectors of der_cjckd8
    ns = n[s_idx]
    coc = (1.0 - ns) / H_CUT
    F = np.exp(-coc ** 2)
    dF = 2.0 * coc / H_CUT
    nd = np.zeros(P)
    dnd = np.zeros_like(dn)
    nd[s_idx] = ns * F
    nd[weak] = n[weak] * F[:, None]
    dnd[s_idx] = F[:, None] * dn[s_idx] * (1.0 + ns * dF)[:, None]
    dnd[weak] = F[:, None, None] * (dn[weak] + dF[:, None, None] * n[weak][:, :, None] * dn[s_idx][:, None, :])
    nd12 = np.sqrt(nd)
    dnd12 = 0.5 * dnd / np.maximum(nd12, 1e-15)[:, None]
    fi = np.sqrt(np.clip(n * (1.0 - n), 0.0, None))
    dfi = np.zeros_like(dn)
    dfi[no1:] = ((1.0 - 2.0 * n[no1:]) / (2.0 * np.maximum(fi[no1:], 1e-15)))[:, None] * dn[no1:]
    YJ, YK = J_MO.T, K_MO.T  # sum_ij D[i, j, k] X[j, i] = sum_ij D[i, j, k] Y[i, j]
    S, W = slice(no1, nb), slice(na, P)

    def blk(u, v, A, B, Y):  # sum_{a in A, b in B} u[a, k] v[b] Y[a, b]
        return u[A].T @ (Y[A, B] @ v[B])

    gJ = 2.0 * dn.T @ (YJ @ n)
    gK = dn.T @ (YK @ n)
    gK += blk(dfi, fi, S, W, YK) + blk(dfi, fi, W, S, YK) + blk(dfi, fi, W, W, YK)
    gK += blk(dnd12, nd12, S, W, YK) - blk(dnd, nd, S, W, YK)
    gK += blk(dnd12, nd12, W, S, YK) - blk(dnd, nd, W, S, YK)
    gK += -blk(dnd12, nd12, W, W, YK) - blk(dnd, nd, W, W, YK)
    # pair blocks G x G (strong first, then its weak orbitals): der_cjckd8
    # overwrites them (C^J: 0; C^K: the sqrt forms) and calcoccg zeroes the
    # diagonals; subtract the generic value computed above, add the actual
    m = block.shape[1]
    Gi = block[:, :, None]
    Gj = block[:, None, :]
    YJb, YKb = YJ[Gi, Gj], YK[Gi, Gj]  # (ndoc, m, m)
    dnb = dn[block]  # (ndoc, m, nv)
    nb_ = n[block]
    gJ -= 2.0 * np.einsum("pak,pb,pab->k", dnb, nb_, YJb)
    # generic C^K derivative in the block: base + the S x W, W x S, W x W terms
    is_w = np.arange(m) > 0  # position 0 is the strong orbital (in S), the rest weak (in W)
    sw = np.outer(~is_w, is_w) | np.outer(is_w, ~is_w)  # S x W or W x S
    ww = np.outer(is_w, is_w)
    gen = np.einsum("pak,pb->pabk", dnb, nb_)
    fib, dfib = fi[block], dfi[block]
    ndb, dndb, nd12b, dnd12b = nd[block], dnd[block], nd12[block], dnd12[block]
    t_fi = np.einsum("pak,pb->pabk", dfib, fib)
    t_12 = np.einsum("pak,pb->pabk", dnd12b, nd12b)
    t_nd = np.einsum("pak,pb->pabk", dndb, ndb)
    gen += (sw | ww)[None, :, :, None] * t_fi
    gen += sw[None, :, :, None] * (t_12 - t_nd) + ww[None, :, :, None] * (-t_12 - t_nd)
    gK -= np.einsum("pabk,pab->k", gen, YKb)
    # actual C^K derivative in the block (der_cjckd8's intra-pair assignments)
    sq = np.sqrt(nb_)
    inv = 1.0 / np.sqrt(np.maximum(nb_, 1e-15))
    act = np.zeros_like(gen)
    act[:, 0, 1:, :] = 0.5 * inv[:, 0, None, None] * sq[:, 1:, None] * dnb[:, 0, None, :]
    act[:, 1:, 0, :] = 0.5 * inv[:, 1:, None] * dnb[:, 1:, :] * sq[:, 0, None, None]
    act[:, 1:, 1:, :] = -0.5 * (dnb[:, 1:, :] * inv[:, 1:, None])[:, :, None, :] * sq[:, None, 1:, None]
    eye = np.eye(m, dtype=bool)
    act[:, eye, :] = 0.0
    gK += np.einsum("pabk,pab->k", act, YKb)
    # diagonals outside the pair blocks (orbitals below no1: the reference's
    # softmax writes pair i's strong row at index i), zeroed by calcoccg
    out = np.ones(P, dtype=bool)
    out[block.ravel()] = False
    if np.any(out):
        o = np.nonzero(out)[0]
        gJ -= 2.0 * dn[o].T @ (n[o] * np.diagonal(YJ)[o])
        gK -= dn[o].T @ (n[o] * np.diagonal(YK)[o])
    g = dn.T @ (2.0 * H_core + np.diagonal(J_MO))
    return g + 2.0 * gJ - 2.0 * gK


def native_occ_ok(p) -> bool:
    """Structures the compiled occupation function covers (closed shell,
    no singly occupied orbitals)."""
    return p.MSpin == 0 and p.nsoc == 0 and p.ndoc >= 1 and p.ncwo >= 1


class OccFunction:
    """E(gamma) and dE/dgamma (calcocce, calcoccg) at fixed J_MO, K_MO,
    H_core from the library's compiled host loop ``gb_occ_energy_grad_f64``:
    one O(nbf5^2) pass instead of numpy's many small array operations.  A call
    returns (E, g), the form ``scipy.optimize.minimize(..., jac=True)`` takes."""

    def __init__(self, J_MO, K_MO, H_core, p):
        from . import _lib

        self._lib = _lib
        self._J = np.ascontiguousarray(J_MO, dtype=np.float64)
        self._K = np.ascontiguousarray(K_MO, dtype=np.float64)
        self._H = np.ascontiguousarray(H_core, dtype=np.float64)
        self._dims = (p.nbf5, p.no1, p.ndoc, p.ncwo)
        self._E = np.zeros(1)
        self._nv = p.nv

    def __call__(self, gamma):
        x = np.ascontiguousarray(gamma, dtype=np.float64)
        g = np.empty(self._nv)
        self._lib.call("gb_occ_energy_grad_f64", x.ctypes.data, self._J.ctypes.data, self._K.ctypes.data,
                       self._H.ctypes.data, *self._dims, self._E.ctypes.data, g.ctypes.data)
        return float(self._E[0]), g

    def energy(self, gamma) -> float:
        x = np.ascontiguousarray(gamma, dtype=np.float64)
        self._lib.call("gb_occ_energy_grad_f64", x.ctypes.data, self._J.ctypes.data, self._K.ctypes.data,
                       self._H.ctypes.data, *self._dims, self._E.ctypes.data, None)
        return float(self._E[0])


def calcocce(gamma, J_MO, K_MO, H_core, p):
    """``pnof.py:994-1001``."""
    n, _ = ocupacion_softmax(gamma, p)
    cj, ck = cjckd8(n, p)
    return calce(n, cj, ck, J_MO, K_MO, H_core, p)


def calcoccg(gamma, J_MO, K_MO, H_core, p):
    """Occupation gradient dE/dgamma (``pnof.py:1004-1033``, closed shell)."""
    n, dn = ocupacion_softmax(gamma, p)
    Dcj, Dck = der_cjckd8(n, dn, p)
    idx = np.arange(p.nbf5)
    Dcj[idx, idx] = 0.0
    Dck[idx, idx] = 0.0
    g = dn.T @ (2.0 * H_core + np.diagonal(J_MO))
    g += 2.0 * np.einsum("ijk,ji->k", Dcj, J_MO)
    g -= 2.0 * np.einsum("ijk,ji->k", Dck, K_MO)
    return g


@functools.lru_cache(maxsize=64)
def _packed_index(nbf: int, nbf5: int):
    """Flat indices of (i, j > i), i < nbf5, row-major: the packed order of y."""
    iu, ju = np.triu_indices(nbf, 1)
    keep = iu < nbf5
    return iu[keep] * nbf + ju[keep], ju[keep] * nbf + iu[keep]


def orbital_gradient(elag, p):
    """Packed 4 (elag - elag^T) over i < nbf5, j > i (``pnof.py:1114-1131``)."""
    ij, ji = _packed_index(p.nbf, p.nbf5)
    e = np.asarray(elag).reshape(-1)
    return 4.0 * (e[ij] - e[ji])


def rotate_orbital(y, C, p):
    """C expm(Y), Y antisymmetric from the packed y (``utils.py:550-565``)."""
    N = p.nbf
    Y = np.zeros((N, N))
    iu, ju = np.triu_indices(N, 1)
    keep = iu < p.nbf5
    Y[iu[keep], ju[keep]] = y
    Y -= Y.T
    return C @ scipy.linalg.expm(Y)


def order_occupations_softmax(C, gamma, p):
    """Sort every strong/weak subspace so that the strong orbital carries the
    largest occupation (``guess.py:77-106``)."""
    C = C.copy()
    gnew = np.zeros(p.nv)
    for s, weak, gam in _pairs(p):
        cols = np.concatenate(([s], weak))
        g = np.concatenate(([0.0], gamma[gam]))
        order = np.argsort(g, kind="stable")[::-1]
        g = g[order] - g.max()
        C[:, cols] = C[:, cols][:, order]
        gnew[gam] = g[1:]
    return C, gnew


def gamma_guess_softmax(p):
    """Starting gammas: every weak occupation 0.001 / ncwo of its pair
    (the value ``utils.py:680-689`` writes)."""
    return np.full(p.nv, np.log(max(0.001 / p.ncwo, 1e-16)) - np.log(0.999))
