"""Parity of the full-ERI path and the AO (Fock) route with the reference.

Tolerance 1e-10 normwise (energies: 1e-10 relative).
"""
import types

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


def _eri(torch, b):
    from pynof_gb300 import ops

    db = ops.to_device(b)
    N, _, Q = db.shape
    B = db.reshape(N * N, Q)
    return (B @ B.T).reshape(N, N, N, N).contiguous()


@pytest.mark.parametrize("name", ["c1", "water"])
def test_full_eri_golden(torch_cuda, name):
    from pynof_gb300 import integrals_full, ops, utils

    g = load_golden(name)
    p = param_for(name)
    p.RI = False
    I = _eri(torch_cuda, g["b"])
    J, K = integrals_full.JKj_Full_GPU(g["C"], I, p)
    assert nrel(J, g["J_full"]) < TOL and nrel(K, g["K_full"]) < TOL
    a, b, c = integrals_full.JKH_MO_Full_GPU(g["C"], g["H"], I, p)
    assert nrel(a, g["J_MO_full"]) < TOL and nrel(b, g["K_MO_full"]) < TOL and nrel(c, g["H_core"]) < TOL
    cj, ck = g["cj12"].copy(), g["ck12"].copy()
    elag, Hmat = utils.computeLagrange2(g["n_soft"], cj, ck, g["C"], g["H"], I, None, p)
    assert nrel(elag, g["elag2_full"]) < TOL and nrel(Hmat, g["Hmat"]) < TOL
    assert np.all(np.diag(cj) == 0) and np.all(np.diag(ck) == 0)


@pytest.mark.parametrize("N,ndoc,ncwo", [(13, 2, 3), (21, 3, 4)])
def test_mo_full_vs_oracle(torch_cuda, N, ndoc, ncwo):
    from oracle import pynof_oracle as orc
    from pynof_gb300 import ops, synthetic

    st = synthetic.Structure(nbf=N, nbfaux=3 * N, ndoc=ndoc, ncwo=ncwo)
    b, C, H, n = synthetic.make_inputs(st, 21 + N)
    I = orc.eri_from_b(b)
    Hm, imo = ops.mo_full(ops.to_device(C), ops.to_device(H), ops.to_device(I), st.nbf5)
    Hr, ir = orc.integrals_mo_full(C, H, I, st.nbf5)
    assert nrel(Hm.cpu().numpy(), Hr) < TOL and nrel(imo.cpu().numpy(), ir) < TOL
    J, K = ops.jkj_full(ops.to_device(C), ops.to_device(I), st.nbf5)
    Jr, Kr = orc.jkj_full(C, I, st.nbf5)
    assert nrel(J.cpu().numpy(), Jr) < TOL and nrel(K.cpu().numpy(), Kr) < TOL


@pytest.fixture(params=sorted(GOLDEN_CASES))
def case(request, torch_cuda):
    name = request.param
    return load_golden(name), param_for(GOLDEN_CASES[name])


def test_fock_lagrange_energy(case):
    from pynof_gb300 import ops, utils

    g, p = case
    cj, ck = g["cj12"].copy(), g["ck12"].copy()
    F = utils.computeF_RC_GPU(g["J_ri"], g["K_ri"], g["n_soft"], g["H"], cj, ck, p)
    assert nrel(F, g["F_rc"]) < TOL
    dC = ops.to_device(g["C"])
    elag = ops.lagrange(ops.to_device(F), dC, p.noptorb)
    assert nrel(elag.cpu().numpy(), g["elag_F"]) < TOL
    E = float(ops.energy_elec(elag, dC, ops.to_device(g["H"]), ops.to_device(g["n_soft"]), p.nbeta, p.nalpha))
    assert abs(E - float(g["E_F"])) < TOL * abs(float(g["E_F"]))


def test_energy1r_both_routes(case):
    from pynof_gb300 import integrals, ops, utils

    g, p = case
    db = ops.to_device(g["b"])
    for mode in ("fp64", "mixed"):
        integrals.set_precision(mode, 6)
        try:
            E, elag, sd, md = utils.ENERGY1r(g["C"], g["n_soft"], g["H"], None, db, g["cj12"].copy(),
                                             g["ck12"].copy(), p)
            assert abs(E - float(g["E1r"])) < TOL * abs(float(g["E1r"]))
            assert nrel(elag, g["elag1r"]) < TOL
            ph = types.SimpleNamespace(**vars(p))
            ph.no1 = p.nbeta
            nh = np.zeros(p.nbf5)
            nh[: p.nbeta] = 1.0
            Eh, elagh, _, _ = utils.ENERGY1r(g["C"], nh, g["H"], None, db, 2 * np.outer(nh, nh), np.outer(nh, nh), ph)
            assert abs(Eh - float(g["E1r_hf"])) < TOL * abs(Eh), mode
            assert nrel(elagh, g["elag1r_hf"]) < TOL, mode
        finally:
            integrals.set_precision("mixed", 6)


@pytest.mark.parametrize("name", ["c1", "water"])
def test_hf_jk_golden(torch_cuda, name):
    """The HF-JK drop-ins against the reference's own outputs."""
    import types as _t

    from pynof_gb300 import integrals, integrals_hf

    g = load_golden(name)
    p = param_for(GOLDEN_CASES[name])
    I = integrals.upload_integrals(np.einsum("mnQ,slQ->mnsl", g["b"], g["b"]), None)[0]
    D = integrals_hf.computeD_HF(g["C"], p)
    assert nrel(D, g["D_hf"]) < 1e-12
    J, K = integrals_hf.computeJK_HF(D, I, None, p)
    assert nrel(J, g["J_hf"]) < 1e-10 and nrel(K, g["K_hf"]) < 1e-10
    pa = _t.SimpleNamespace(**vars(p))
    pa.nalpha = p.nbeta + 2
    Da, Ja, Ka = integrals_hf.computeJKalpha_HF(g["C"], I, None, pa)
    assert nrel(Da, g["Da_hf"]) < 1e-12
    assert nrel(Ja, g["Ja_hf"]) < 1e-10 and nrel(Ka, g["Ka_hf"]) < 1e-10
    assert nrel(integrals_hf.computeDalpha_HF(g["C"], pa), g["Da_hf"]) < 1e-12


@pytest.mark.parametrize("name", ["c1", "water"])
def test_post_nof_transforms_golden(torch_cuda, name):
    """compute_iajb / compute_pqrt drop-ins against the reference's outputs."""
    from pynof_gb300 import integrals, integrals_full

    g = load_golden(name)
    p = param_for(GOLDEN_CASES[name])
    I = integrals.upload_integrals(np.einsum("mnQ,slQ->mnsl", g["b"], g["b"]), None)[0]
    assert nrel(integrals_full.compute_iajb(g["C"], I, None, p), g["iajb"]) < 1e-10
    assert nrel(integrals_full.compute_pqrt(g["C"], I, None, p), g["pqrt"]) < 1e-10



def _open_shell_param(**over):
    import json
    import os

    from conftest import GOLDEN
    from pynof_gb300 import synthetic

    with open(os.path.join(GOLDEN, "golden_meta.json")) as f:
        st = synthetic.Structure(**json.load(f)["open_shell"]["sizes"])
    for k, v in over.items():
        setattr(st, k, v)
    return st


def test_open_shell_fock_route(torch_cuda):
    """computeF_RO (utils.py:172-246), computeLagrange, computeE_elec (both
    HighSpin settings) and ENERGY1r's no1 > 0, MSpin != 0 route, RI and
    full ERI, FP64 and split products, against the reference's outputs."""
    from pynof_gb300 import integrals, ops, utils

    g = load_golden("open_shell")
    p = _open_shell_param()
    cj, ck = g["cj12"].copy(), g["ck12"].copy()
    F = utils.computeF_RO_GPU(g["J_ri"], g["K_ri"], g["n"], g["H"], cj, ck, p)
    assert nrel(F, g["F_ro"]) < TOL
    assert np.array_equal(cj, g["cj12_zeroed"]) and np.array_equal(ck, g["ck12_zeroed"])
    dC, dH, dn = ops.to_device(g["C"]), ops.to_device(g["H"]), ops.to_device(g["n"])
    elag = ops.lagrange(ops.to_device(F), dC, p.noptorb)
    assert nrel(elag.cpu().numpy(), g["elag_F"]) < TOL
    for hs, key in ((False, "E_F"), (True, "E_F_highspin")):
        E = float(ops.energy_elec(elag, dC, dH, dn, p.nbeta, p.nalpha, hs))
        assert abs(E - float(g[key])) < TOL * abs(float(g[key])), key
    db = ops.to_device(g["b"])
    I = integrals.upload_integrals(np.einsum("mnQ,slQ->mnsl", g["b"], g["b"]), None)[0]
    pf = _open_shell_param(RI=False)
    for mode in ("fp64", "mixed"):
        integrals.set_precision(mode, 6)
        try:
            for pp, ints in ((p, (None, db)), (pf, (I, None))):
                E1, el1, sd, md = utils.ENERGY1r(g["C"], g["n"], g["H"], ints[0], ints[1], g["cj12"].copy(),
                                                 g["ck12"].copy(), pp)
                assert abs(E1 - float(g["E1r"])) < TOL * abs(E1), (mode, pp.RI)
                assert nrel(el1, g["elag1r"]) < TOL, (mode, pp.RI)
        finally:
            integrals.set_precision("mixed", 6)
