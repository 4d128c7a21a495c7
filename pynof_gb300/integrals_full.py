"""Drop-in mirror of PyNOF's full-ERI GPU functions (``pynof/integrals.py``).

``I`` is the device-resident (nbf, nbf, nbf, nbf) float64 tensor; host inputs
are uploaded per call and results return as host numpy arrays, except
``Integrals_MO_Full_GPU`` which returns device tensors like the reference.
"""
from __future__ import annotations

from . import ops
from .integrals import as_device, to_host


def JKj_Full_GPU(C, I, p):
    """J, K (nbf5, nbf, nbf) -- ``pynof/integrals.py:221-231``."""
    return to_host(*ops.jkj_full(as_device(C), as_device(I), p.nbf5))


def JKH_MO_Full_GPU(C, H, I, p):
    """J_MO, K_MO, H_core -- ``pynof/integrals.py:365-380``."""
    return to_host(*ops.jkh_mo_full(as_device(C), as_device(H), as_device(I), p.nbf5))


def Integrals_MO_Full_GPU(C, H, I, p):
    """H_mat (nbf, nbf5), I_MO (nbf, nbf5, nbf5, nbf5) on the device --
    ``pynof/integrals.py:693-698``."""
    return ops.mo_full(as_device(C), as_device(H), as_device(I), p.nbf5)


def iajb_Full_GPU(C, I, p):
    """``pynof/integrals.py:626-638``: (ia|jb) over occupied i, j in
    [no1, nalpha) and virtual a, b in [nalpha, nbf); host numpy out."""
    occ, vir = (p.no1, p.nalpha), (p.nalpha, p.nbf)
    return to_host(ops.mo4_full(as_device(C), as_device(I), occ, vir, occ, vir))


def compute_iajb(C, I, b_mnl, p):
    """``pynof/integrals.py:601-608`` (the GPU branch)."""
    return iajb_Full_GPU(C, I, p)


def pqrt_Full_GPU(C, I, p):
    """``pynof/integrals.py:657-660``: the full four-index MO transform."""
    a = (0, p.nbf)
    return to_host(ops.mo4_full(as_device(C), as_device(I), a, a, a, a))


def compute_pqrt(C, I, b_mnl, p):
    """``pynof/integrals.py:641-648`` (the GPU branch)."""
    return pqrt_Full_GPU(C, I, p)

