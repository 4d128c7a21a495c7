"""Drop-in ``occoptr`` with the occupation optimiser on the device.

``pynof/minimization.py:77-97`` forms J_MO, K_MO, H_core at the orbitals
(``computeJKH_MO``), minimises the occupation energy over gamma with
``scipy.optimize.minimize(calcocce, gamma, jac=calcoccg, method="CG")`` and
returns ``(E, nit, success, gamma, n, cj12, ck12)``.  Here J_MO, K_MO, H_core
stay on the device and the minimisation is one CUDA graph
(:class:`ops.OccMinimizer`, scipy's CG steps); gamma, n, C^J, C^K and the
result come back to the host in one synchronisation.  Host numpy out, as the
reference returns.

Covers the structures the device optimiser handles -- GNOF (``ipnof`` 8) with
softmax occupations, closed shell, ``occupation_optimizer == "CG"``,
occupations not frozen; :mod:`pynof_gb300.install` routes every other case
to the reference's own ``occoptr``.
"""
from __future__ import annotations

import threading

import torch

from . import integrals, nof, ops

_lock = threading.Lock()
_minimizers: dict = {}


def device_ok(p) -> bool:
    """The structures and settings ``occoptr`` runs on the device."""
    return (getattr(p, "gpu", False) and getattr(p, "ipnof", None) == 8
            and getattr(p, "occ_method", None) == "Softmax"
            and getattr(p, "occupation_optimizer", "CG") == "CG"
            and not getattr(p, "freeze_occ", False) and p.ndoc > 0 and nof.native_occ_ok(p))


def minimizer(p) -> ops.OccMinimizer:
    """One optimiser (workspace and cached graph) per device and structure."""
    dev = torch.cuda.current_device()
    key = (dev, p.nbf5, p.no1, p.ndoc, p.ncwo)
    with _lock:
        om = _minimizers.get(key)
        if om is None:
            om = ops.OccMinimizer(p.nbf5, p.no1, p.ndoc, p.ncwo, torch.device("cuda", dev))
            _minimizers[key] = om
        return om


def occoptr(gamma, C, H, I, b_mnl, p):
    """``minimization.py:77-97`` with J_MO, K_MO, H_core on the device and the
    CG over gamma as one device graph."""
    if p.RI:
        J, K, Hc = integrals.jkh_mo_ri_device(C, H, b_mnl, p.nbf5)
    else:
        J, K, Hc = ops.jkh_mo_full(integrals.as_device(C), integrals.as_device(H), integrals.as_device(I), p.nbf5)
    om = minimizer(p)
    with _lock:
        gam, res, n, cj12, ck12 = om.minimize(integrals.as_device(gamma), J, K, Hc)
        gam, res, n, cj12, ck12 = integrals.to_host(gam, res, n, cj12, ck12)
    if res[3] < 0:
        raise RuntimeError("occupation minimiser reached its evaluation cap")
    return float(res[0]), int(res[1]), bool(res[3] == 1.0), gam, n, cj12, ck12

