"""Drop-in mirror of PyNOF's HF-JK helpers (``pynof/integrals.py:490-562``):
the closed-shell and singly-occupied densities and their J, K from the
4-index tensor, on the device in FP64.  Host numpy in, host numpy out, as the
reference's ``*_GPU`` functions return after ``.get()``.

The reference computes these with the 4-index tensor only (its RI branches
are commented out), so ``b_mnl`` is accepted and ignored, as there.
"""
from __future__ import annotations

from . import ops
from .integrals import as_device, to_host


def computeD_HF(C, p):
    """``integrals.py:493-500``: D = C[:, :nbeta] C[:, :nbeta]^T."""
    return to_host(ops.density_hf(as_device(C), 0, p.nbeta))


def computeDalpha_HF(C, p):
    """``integrals.py:503-510``: D = C[:, nbeta:nalpha] C[:, nbeta:nalpha]^T."""
    return to_host(ops.density_hf(as_device(C), p.nbeta, p.nalpha))


def JK_HF_Full_GPU(D, I, p):
    """``integrals.py:537-543``: J = einsum("ls,mnsl->mn"), K = einsum("nl,mnsl->ms")
    for a symmetric D; I resident on the device."""
    J, K = ops.jk_hf_full(as_device(D), as_device(I))
    return to_host(J, K)


def computeJK_HF(D, I, b_mnl, p):
    """``integrals.py:513-525`` (the GPU branch)."""
    return JK_HF_Full_GPU(D, I, p)


def JKalpha_HF_Full_GPU(C, I, p):
    """``integrals.py:557-562``: the singly-occupied density and its J, K."""
    D = ops.density_hf(as_device(C), p.nbeta, p.nalpha)
    J, K = ops.jk_hf_full(D, as_device(I))
    return to_host(D, J, K)


def computeJKalpha_HF(C, I, b_mnl, p):
    """``integrals.py:546-554`` (the GPU branch)."""
    return JKalpha_HF_Full_GPU(C, I, p)
