"""Parity of the FP64 RI path (CUDA, through the C ABI) with the reference.

Tolerance: 1e-10 normwise relative (max|gpu - ref| / max|ref|), the bar the
plain FP64 path must meet against PyNOF's own numpy functions.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, nrel, param_for

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(params=sorted(GOLDEN_CASES))
def case(request, torch_cuda):
    from pynof_gb300 import ops

    name = request.param
    g = load_golden(name)
    p = param_for(GOLDEN_CASES[name])
    dev = {k: ops.to_device(g[k]) for k in ("b", "C", "H")}
    return g, p, dev


def test_jkj_ri(case):
    from pynof_gb300 import ops

    g, p, d = case
    J, K = ops.jkj_ri(d["C"], d["b"], p.nbf5)
    assert nrel(J.cpu().numpy(), g["J_ri"]) < TOL
    assert nrel(K.cpu().numpy(), g["K_ri"]) < TOL


def test_jkh_mo_ri(case):
    from pynof_gb300 import ops

    g, p, d = case
    a, b, c = ops.jkh_mo_ri(d["C"], d["H"], d["b"], p.nbf5)
    assert nrel(a.cpu().numpy(), g["J_MO_ri"]) < TOL
    assert nrel(b.cpu().numpy(), g["K_MO_ri"]) < TOL
    assert nrel(c.cpu().numpy(), g["H_core"]) < TOL


def test_mo_ri(case):
    from pynof_gb300 import ops

    g, p, d = case
    Hmat, bmo = ops.mo_ri(d["C"], d["H"], d["b"], p.nbf5)
    assert nrel(Hmat.cpu().numpy(), g["Hmat"]) < TOL
    assert nrel(bmo.cpu().numpy(), g["b_MO"]) < TOL


def test_lagrange2_ri(case):
    from pynof_gb300 import ops

    g, p, d = case
    n = ops.to_device(g["n_soft"])
    cj = ops.to_device(g["cj12"])
    ck = ops.to_device(g["ck12"])
    elag, Hmat = ops.lagrange2_ri(d["C"], d["H"], d["b"], n, cj, ck, p.nbf5, p.nbeta, p.nalpha)
    assert nrel(elag.cpu().numpy(), g["elag2_ri"]) < TOL
    assert nrel(Hmat.cpu().numpy(), g["Hmat"]) < TOL


def test_symmetry_check(case):
    from pynof_gb300 import ops

    g, p, d = case
    assert ops.check_symmetric(d["b"]) == 0.0


@pytest.mark.parametrize("N,Q,ndoc,ncwo,seed", [(5, 7, 1, 1, 11), (67, 131, 6, 4, 12), (130, 260, 13, 4, 13),
                                                 (64, 64, 8, 7, 14)])
def test_odd_sizes_vs_oracle(torch_cuda, N, Q, ndoc, ncwo, seed):
    """Sizes that are not multiples of the 64 x 64 x 16 tiles, P = N and P < N."""
    from oracle import pynof_oracle as orc
    from pynof_gb300 import ops, synthetic

    st = synthetic.Structure(nbf=N, nbfaux=Q, ndoc=ndoc, ncwo=ncwo)
    b, C, H, n = synthetic.make_inputs(st, seed)
    P = st.nbf5
    db, dC, dH = ops.to_device(b), ops.to_device(C), ops.to_device(H)
    J, K = ops.jkj_ri(dC, db, P)
    Jr, Kr = orc.jkj_ri(C, b, P)
    assert nrel(J.cpu().numpy(), Jr) < TOL and nrel(K.cpu().numpy(), Kr) < TOL
    a, bb, c = ops.jkh_mo_ri(dC, dH, db, P)
    ar, br, cr = orc.jkh_mo_ri(C, H, b, P)
    assert nrel(a.cpu().numpy(), ar) < TOL and nrel(bb.cpu().numpy(), br) < TOL and nrel(c.cpu().numpy(), cr) < TOL
    cj = np.abs(np.random.default_rng(seed).standard_normal((P, P)))
    ck = np.abs(np.random.default_rng(seed + 1).standard_normal((P, P)))
    el, Hm = ops.lagrange2_ri(dC, dH, db, ops.to_device(n), ops.to_device(cj), ops.to_device(ck), P, st.nbeta,
                              st.nalpha)
    elr, Hmr = orc.lagrange2(n, cj.copy(), ck.copy(), C, H, None, b, st)
    assert nrel(el.cpu().numpy(), elr) < TOL and nrel(Hm.cpu().numpy(), Hmr) < TOL


def test_errors_are_raised(torch_cuda):
    from pynof_gb300 import _lib, ops

    b = torch_cuda.zeros((4, 4, 3), dtype=torch_cuda.float64, device="cuda")
    C = torch_cuda.zeros((4, 4), dtype=torch_cuda.float64, device="cuda")
    with pytest.raises(_lib.GBError):
        ops.jkj_ri(C, b, 5)  # nbf5 > nbf
    with pytest.raises(ValueError):
        ops.jkj_ri(C[:3, :3].contiguous(), b, 2)
