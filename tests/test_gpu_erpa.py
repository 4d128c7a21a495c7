"""ERPA's MO integrals on the RI route (postpnof.py:1402-1406) against the
oracle: h and (pq|sl) = sum_R b_pqR b_slR, FP64 (1e-12) and split (1e-10)."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, nrel, param_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("mode,tol", [("fp64", 1e-12), ("mixed", 1e-10)])
@pytest.mark.parametrize("name", sorted(GOLDEN_CASES))
def test_erpa_mo_integrals_ri(torch_cuda, name, mode, tol):
    from oracle import pynof_oracle as orc
    from pynof_gb300 import integrals

    g = load_golden(name)
    p = param_for(GOLDEN_CASES[name])
    h_ref, I_ref = orc.erpa_mo_integrals_ri(g["C"], g["H"], g["b"], p.nbf5)
    old = dict(integrals.PRECISION)
    try:
        integrals.set_precision(mode, 6)
        h, I = integrals.erpa_mo_integrals_ri(g["C"], g["H"], g["b"], p)
    finally:
        integrals.set_precision(old["mode"], old["nslices"])
    assert nrel(h, h_ref) < 1e-12
    assert nrel(I, I_ref) < tol
