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


def ocupacion_softmax(gamma, p):
    """Occupations n (nbf5,) and dn/dgamma (nbf5, nv) from the softmax
    parameterisation (``pnof.py:770-809``): each strong orbital and its weak
    partners share one softmax with a zero logit for the strong orbital."""
    n = np.zeros(p.nbf5)
    dn = np.zeros((p.nbf5, p.nv))
    n[p.no1 + p.ndoc: p.no1 + p.ndns] = 1.0 if p.HighSpin else 0.5
    for i, (_, weak, gam) in enumerate(_pairs(p)):
        x = gamma[gam]
        top = x.max() if len(x) else 0.0
        if top < 700.0:
            e = np.exp(x)
            den = 1.0 + e.sum()
            ns = 1.0 / den
            nw = e / den
        else:
            # logits a line search pushed past exp's range: the same softmax,
            # shifted by its largest logit
            e = np.exp(x - top)
            den = np.exp(-top) + e.sum()
            ns = np.exp(-top) / den
            nw = e / den
        # the reference writes the strong occupation at index i (pnof.py:793)
        n[i] = ns
        n[weak] = nw
        dn[i, gam] = -ns * nw
        dn[np.ix_(weak, gam)] = np.diag(nw) - np.outer(nw, nw)
    return n, dn


def cjckd8(n, p):
    """GNOF coefficients C^J, C^K (nbf5, nbf5) (``pnof.py:350-422``)."""
    no1, nb, na = p.no1, p.nbeta, p.nalpha
    nd = np.zeros_like(n)
    for s, weak, _ in _pairs(p):
        F = np.exp(-((1.0 - n[s]) / H_CUT) ** 2)
        nd[s] = n[s] * F
        nd[weak] = n[weak] * F
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
    for s, weak, _ in _pairs(p):
        cj[s, weak] = 0.0
        cj[weak, s] = 0.0
        cj[np.ix_(weak, weak)] = 0.0
        ck[s, weak] = np.sqrt(n[s] * n[weak])
        ck[weak, s] = np.sqrt(n[s] * n[weak])
        ck[np.ix_(weak, weak)] = -np.sqrt(np.outer(n[weak], n[weak]))
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
    ck12 are zeroed in place, as in the reference."""
    P = p.nbf5
    np.fill_diagonal(cj12, 0.0)
    np.fill_diagonal(ck12, 0.0)
    dj = np.diagonal(J_MO)
    E = 2.0 * np.dot(n, H_core) + np.dot(n[: p.nbeta], dj[: p.nbeta]) + np.dot(n[p.nalpha: P], dj[p.nalpha: P])
    return E + np.sum(cj12 * J_MO.T) - np.sum(ck12 * K_MO.T)


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
