"""Drop-in mirror of PyNOF's GPU integral functions.

Same names, argument order and return types as the functions PyNOF dispatches
to when ``p.gpu`` is set (``pynof/integrals.py``), so that an installer can
rebind them in the ``pynof`` namespace:

* host inputs (``C``, ``H``, ``n``, ``cj12``, ``ck12``) are numpy float64 arrays
  of any strides and are uploaded per call, like the reference's ``cp.array``;
* ``b_mnl`` / ``I`` are device-resident (a float64 CUDA tensor, uploaded once
  by :func:`upload_integrals`); numpy inputs are accepted and uploaded per call;
* results come back as host numpy arrays, like the reference's ``.get()``,
  except where the reference returns device arrays (``Integrals_MO_*_GPU``
  return torch CUDA tensors where the reference returns cupy arrays).

All arithmetic runs in ``libpynof_gb300.so``; there is no CPU fallback.
"""
from __future__ import annotations

import threading
import weakref

import numpy as np
import torch

from . import ops

#: Arithmetic of the device path: "fp64" (DMMA) or "mixed" (tcgen05 split
#: products; nslices=6 bf16 digit slices agree with FP64 to ~1e-11, nslices=2
#: is bf16x3, nslices=ops.SPLIT_TF32X3 is tf32x3).
PRECISION = {"mode": "mixed", "nslices": 6}

_prep_lock = threading.Lock()
# id(b) -> (weakref to b, b._version, {nslices: PreparedRI}); entries die with b
_prepared: dict = {}


def set_precision(mode: str, nslices: int = 6) -> None:
    if mode not in ("fp64", "mixed"):
        raise ValueError(f"unknown precision mode {mode!r}")
    if not (1 <= nslices <= 6 or nslices == ops.SPLIT_TF32X3):
        raise ValueError(f"nslices must be in [1, 6] or ops.SPLIT_TF32X3 ({ops.SPLIT_TF32X3})")
    PRECISION["mode"] = mode
    PRECISION["nslices"] = nslices


def prepared(b: torch.Tensor, nslices: int) -> ops.PreparedRI:
    """The sliced RI factor for ``b`` (built once per tensor and slice count)."""
    key = id(b)
    with _prep_lock:
        ent = _prepared.get(key)
        if ent is not None and (ent[0]() is not b or ent[1] != b._version):
            ent = None
        if ent is not None and nslices in ent[2]:
            return ent[2][nslices]
        prep = ops.PreparedRI(b, nslices)
        if ent is None:
            ref = weakref.ref(b, lambda _r, k=key: _prepared.pop(k, None))
            ent = (ref, b._version, {})
            _prepared[key] = ent
        ent[2][nslices] = prep
        return prep


def as_device(x) -> torch.Tensor:
    if isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == torch.float64 and x.is_contiguous():
        return x
    return ops.to_device(x)


def to_host(*tensors):
    """Copy device tensors into pinned host memory and return numpy arrays;
    raise GBError if the device status word reports a failed split-product
    kernel or a non-finite operand.

    Pinned blocks come from torch's caching host allocator, so repeated calls
    of the same size reuse the same page-locked memory once the caller drops
    the previous result."""
    outs = []
    for t in tensors:
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t, non_blocking=True)
        outs.append(h)
    torch.cuda.current_stream().synchronize()
    # a split-product kernel that gave up, or a non-finite operand, must not
    # hand back unwritten memory as results
    ops.check_device_status()
    res = tuple(h.numpy() for h in outs)
    return res if len(res) > 1 else res[0]


def upload_integrals(I, b_mnl, check_symmetry: bool = True):
    """Device copies of the ERI tensor(s), the replacement for the ``cp.array``
    upload at the end of ``compute_integrals`` (``pynof/integrals.py:51-53``)."""
    dI = as_device(I) if I is not None and np.size(I) else I
    db = None
    if b_mnl is not None and np.size(b_mnl):
        db = as_device(b_mnl)
        if check_symmetry:
            asym = ops.check_symmetric(db)
            if asym != 0.0:
                raise ValueError(f"b_mnl is not symmetric in (m, n) (max |b - b^T| = {asym:.3e}); "
                                 "the RI kernels require the exact symmetry PyNOF's b_mnl has")
    return dI, db


# ---------------------------------------------------------------------------
# A1  computeJKj
# ---------------------------------------------------------------------------
def jkj_ri_device(C, b_mnl, nbf5):
    """J, K as CUDA tensors with the arithmetic selected by ``PRECISION``."""
    dC, db = as_device(C), as_device(b_mnl)
    if PRECISION["mode"] == "mixed":
        return ops.jkj_ri_mixed(dC, prepared(db, PRECISION["nslices"]), nbf5)
    return ops.jkj_ri(dC, db, nbf5)


def JKj_RI_GPU(C, b_mnl, p):
    """J, K (nbf5, nbf, nbf) -- ``pynof/integrals.py:234-245``.  On the tensor
    cores the copies to the host overlap the build: after T is formed, J and K
    are formed over alternating ranges of 128 orbitals and each range is
    copied as soon as it is done."""
    if PRECISION["mode"] == "mixed":
        db = as_device(b_mnl)
        return ops.jkj_ri_mixed_host(as_device(C), prepared(db, PRECISION["nslices"]), p.nbf5)
    return to_host(*jkj_ri_device(C, b_mnl, p.nbf5))


def computeJKj(C, I, b_mnl, p):
    """Dispatcher of ``pynof/integrals.py:172-191`` for the device path."""
    if p.RI:
        return JKj_RI_GPU(C, b_mnl, p)
    from . import integrals_full

    return integrals_full.JKj_Full_GPU(C, I, p)


# ---------------------------------------------------------------------------
# A3  computeJKH_MO
# ---------------------------------------------------------------------------
def jkh_mo_ri_device(C, H, b_mnl, nbf5):
    """J_MO, K_MO, H_core as CUDA tensors with the arithmetic of ``PRECISION``."""
    dC, dH, db = as_device(C), as_device(H), as_device(b_mnl)
    if PRECISION["mode"] == "mixed":
        return ops.jkh_mo_ri_mixed(dC, dH, prepared(db, PRECISION["nslices"]), nbf5)
    return ops.jkh_mo_ri(dC, dH, db, nbf5)


def JKH_MO_RI_GPU(C, H, b_mnl, p):
    """J_MO, K_MO (nbf5, nbf5), H_core (nbf5,) -- ``pynof/integrals.py:383-399``."""
    return to_host(*jkh_mo_ri_device(C, H, b_mnl, p.nbf5))


def computeJKH_MO(C, H, I, b_mnl, p):
    """Dispatcher of ``pynof/integrals.py:307-326`` for the device path."""
    if p.RI:
        return JKH_MO_RI_GPU(C, H, b_mnl, p)
    from . import integrals_full

    return integrals_full.JKH_MO_Full_GPU(C, H, I, p)


# ---------------------------------------------------------------------------
# A5  JKH_MO_tmp / Integrals_MO_RI
# ---------------------------------------------------------------------------
def Integrals_MO_RI_GPU(C, H, b_mnl, p):
    """H_mat (nbf, nbf5), b_MO (nbf, nbf5, naux) as CUDA tensors --
    ``pynof/integrals.py:709-714`` (which returns device arrays too)."""
    return ops.mo_ri(as_device(C), as_device(H), as_device(b_mnl), p.nbf5)


def JKH_MO_tmp(C, H, I, b_mnl, p):
    """Dispatcher of ``pynof/integrals.py:665-682`` for the device path."""
    if p.RI:
        return Integrals_MO_RI_GPU(C, H, b_mnl, p)
    from . import integrals_full

    return integrals_full.Integrals_MO_Full_GPU(C, H, I, p)


# ---------------------------------------------------------------------------
# The RI factor itself (compute_integrals, integrals.py:35-49)
# ---------------------------------------------------------------------------
def metric_power(metric, alpha: float = -0.5, cutoff: float = 1.0e-14):
    """The metric power compute_integrals takes from psi4
    (``metric.power(-0.5, 1.0e-14)``, ``integrals.py:45``; psi4 is a conda
    dependency the reference does not pin): eigendecomposition of the
    symmetric metric; for a negative power, eigenvalues whose magnitude is
    below ``cutoff`` times the largest are dropped (their power is zero), the
    others are raised to ``alpha``.  Host FP64 (LAPACK): the metric inverse
    square root stays in FP64 on every precision form of the path."""
    a, V = np.linalg.eigh(np.asarray(metric, dtype=np.float64))
    amax = max(abs(a[0]), abs(a[-1])) if a.size else 0.0
    keep = ~((alpha < 0.0) & (np.abs(a) < cutoff * amax))
    pw = np.zeros_like(a)
    with np.errstate(all="ignore"):
        pw[keep] = np.power(a[keep], alpha)
    pw[~np.isfinite(pw)] = 0.0
    return (V * pw) @ V.T


def compute_b_mnl(mnk, metric, nslices: int | None = None, metric_is_power: bool = False):
    """b_mnl = einsum("mnk,kl->mnl", mnk, metric^(-1/2)) (``integrals.py:41-49``)
    with the three-centre integrals mnk (nbf, nbf, naux) as psi4 returns them
    (squeezed): the metric power on the host, the contraction on the device
    (FP64 DMMA, or the split-product tensor-core GEMM with ``nslices``).
    Returns the device tensor (resident, as ``cp.array(b_mnl)`` at ``:53``)."""
    M = np.asarray(metric, dtype=np.float64) if metric_is_power else metric_power(metric)
    return ops.ri_factor(as_device(mnk), as_device(M), nslices)


# ---------------------------------------------------------------------------
# ERPA's MO integrals, RI route (postpnof.py:1402-1406, inline there)
# ---------------------------------------------------------------------------
def erpa_mo_integrals_ri(C, H, b_mnl, p):
    """h = C_p^T H C_p (nbf5, nbf5) and (pq|sl) = sum_R b_pqR b_slR
    (nbf5, nbf5, nbf5, nbf5) with b_pql = sum_mn C_mp C_nq b_mnl, p, q < nbf5
    (``postpnof.py:1402-1406``), on the device: the MO transform of
    computeLagrange2 (A5) and one GEMM over R, FP64 or split per ``PRECISION``.
    Host numpy out (the reference ``.get()``s I)."""
    P = p.nbf5
    dC, dH, db = as_device(C), as_device(H), as_device(b_mnl)
    Hmat, bMO = ops.mo_ri(dC, dH, db, P)
    Q = bMO.shape[2]
    bpq = bMO[:P].reshape(P * P, Q).contiguous()
    if PRECISION["mode"] == "mixed":
        I = ops.dgemm_mixed(bpq, bpq, PRECISION["nslices"])
    else:
        I = ops.dgemm_f64(bpq, bpq)
    return to_host(Hmat[:P].contiguous(), I.view(P, P, P, P))

