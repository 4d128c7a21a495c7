"""Drop-in mirror of PyNOF's Fock / Lagrangian / energy functions
(``pynof/utils.py``) for the device path.

Side effects follow the reference: ``computeLagrange2``, ``computeF_RC_GPU``
and ``computeF_RO_GPU`` zero the diagonals of the caller's ``cj12`` / ``ck12``
in place (``utils.py:46,51,77,81,120,138,269-270``).  For open shells
(MSpin != 0) ``ENERGY1r``'s no1 > 0 route takes the restricted open-shell
Fock (``computeF_RO``), and ``computeLagrange2`` returns a zero Lagrangian
exactly as the reference does.
"""
from __future__ import annotations

import numpy as np
import torch

from . import ops
from .integrals import PRECISION, as_device, jkj_ri_device, prepared, to_host


def _zero_diag(a, start=0):
    if isinstance(a, np.ndarray):
        np.fill_diagonal(a[start:, start:], 0.0)


def computeLagrange2_device(n, cj12, ck12, C, H, I, b_mnl, p):
    """elag (nbf, nbf), Hmat (nbf, nbf5) as CUDA tensors."""
    dC, dH = as_device(C), as_device(H)
    dn, dcj, dck = as_device(n), as_device(cj12), as_device(ck12)
    if p.MSpin != 0:
        N = dC.shape[0]
        Hmat = ops.mo_ri(dC, dH, as_device(b_mnl), p.nbf5)[0] if p.RI else ops.mo_full(dC, dH, as_device(I), p.nbf5)[0]
        return torch.zeros((N, N), dtype=torch.float64, device=dC.device), Hmat
    if p.RI:
        db = as_device(b_mnl)
        if PRECISION["mode"] == "mixed":
            return ops.lagrange2_ri_mixed(dC, dH, prepared(db, PRECISION["nslices"]), dn, dcj, dck, p.nbf5, p.nbeta,
                                          p.nalpha)
        return ops.lagrange2_ri(dC, dH, db, dn, dcj, dck, p.nbf5, p.nbeta, p.nalpha)
    return ops.lagrange2_full(dC, dH, as_device(I), dn, dcj, dck, p.nbf5, p.nbeta, p.nalpha)


def computeLagrange2(n, cj12, ck12, C, H, I, b_mnl, p):
    """elag, Hmat (host numpy) -- ``pynof/utils.py:262-382``."""
    _zero_diag(cj12)
    _zero_diag(ck12)
    return to_host(*computeLagrange2_device(n, cj12, ck12, C, H, I, b_mnl, p))


def computeF_RC_GPU(J, K, n, H, cj12, ck12, p):
    """F (nbf5, nbf, nbf) host numpy -- ``pynof/utils.py:58-84``."""
    ini = p.no1 if p.no1 > 1 else 0
    _zero_diag(cj12, ini)
    _zero_diag(ck12, ini)
    F = ops.fock_rc(as_device(J), as_device(K), as_device(n), as_device(H), as_device(cj12), as_device(ck12),
                    p.nbeta, p.nalpha, p.no1)
    return to_host(F)


def computeF_RC_driver(J, K, n, H, cj12, ck12, p):
    """``pynof/utils.py:15-22`` for the device path."""
    return computeF_RC_GPU(J, K, n, H, cj12, ck12, p)


def computeF_RO_GPU(J, K, n, H, cj12, ck12, p):
    """F (nbf5, nbf, nbf) host numpy, restricted open shell --
    ``pynof/utils.py:172-246``."""
    ini = p.no1 if p.no1 > 1 else 0
    _zero_diag(cj12, ini)
    _zero_diag(ck12, ini)
    F = ops.fock_ro(as_device(J), as_device(K), as_device(n), as_device(H), as_device(cj12), as_device(ck12),
                    p.nbeta, p.nalpha, p.no1)
    return to_host(F)


def computeF_RO_driver(J, K, n, H, cj12, ck12, p):
    """``pynof/utils.py:87-94`` for the device path."""
    return computeF_RO_GPU(J, K, n, H, cj12, ck12, p)


def rotate_orbital(y, C, p):
    """``pynof/utils.py:550-565``: C expm(Y) from the packed step y, on the
    device in FP64 (the reference builds Y in a Python loop and calls
    scipy.linalg.expm).  Host numpy in, host numpy out."""
    Cd = as_device(C)
    yd = as_device(np.asarray(y, dtype=np.float64).reshape(-1))
    return to_host(ops.rotate_orbital(yd, Cd, p.nbf5))


def computeLagrangeConvergency(elag):
    """sumdiff, maxdiff of |elag - elag^T| -- ``pynof/utils.py:405-411``."""
    d = np.abs(elag - elag.T)
    return d.sum(), d.max()


def energy1r_device(C, n, H, I, b_mnl, cj12, ck12, p):
    """E (float), elag (CUDA tensor) of ENERGY1r with every contraction on the device."""
    dC, dH, dn = as_device(C), as_device(H), as_device(n)
    if p.no1 == 0:
        elag, Hmat = computeLagrange2_device(n, cj12, ck12, C, H, I, b_mnl, p)
        P = p.nbf5
        E = torch.trace(elag[:P, :P]) + torch.dot(dn[:P], torch.diagonal(Hmat)[:P])
        return float(E), elag
    ini = p.no1 if p.no1 > 1 else 0
    _zero_diag(cj12, ini)
    _zero_diag(ck12, ini)
    if p.RI:
        J, K = jkj_ri_device(dC, b_mnl, p.nbf5)
    else:
        J, K = ops.jkj_full(dC, as_device(I), p.nbf5)
    fock = ops.fock_rc if p.MSpin == 0 else ops.fock_ro
    F = fock(J, K, dn, dH, as_device(cj12), as_device(ck12), p.nbeta, p.nalpha, p.no1)
    elag = ops.lagrange(F, dC, p.noptorb)
    E = ops.energy_elec(elag, dC, dH, dn, p.nbeta, p.nalpha, p.HighSpin)
    return float(E), elag


def ENERGY1r(C, n, H, I, b_mnl, cj12, ck12, p):
    """E, elag (host), sumdiff, maxdiff -- ``pynof/utils.py:414-431``."""
    E, elag = energy1r_device(C, n, H, I, b_mnl, cj12, ck12, p)
    elag = to_host(elag)
    sumdiff, maxdiff = computeLagrangeConvergency(elag)
    return E, elag, sumdiff, maxdiff
