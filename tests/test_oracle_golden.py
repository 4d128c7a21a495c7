"""The CPU oracle agrees with PyNOF's own outputs (golden fixtures).

The fixtures were produced by running the reference functions
(``tests/golden/make_golden.py``); the oracle is an independent numpy
restatement.  Agreement is required to 1e-12 normwise (BLAS summation order is
the only difference).
"""
import json
import os
import types

import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_CASES, load_golden, nrel, param_for
from oracle import pynof_oracle as orc

TOL = 1e-12


@pytest.fixture(params=sorted(GOLDEN_CASES))
def case(request):
    name = request.param
    return name, load_golden(name), param_for(GOLDEN_CASES[name])


def test_jkj_ri(case):
    _, g, p = case
    J, K = orc.jkj_ri(g["C"], g["b"], p.nbf5)
    assert nrel(J, g["J_ri"]) < TOL
    assert nrel(K, g["K_ri"]) < TOL


def test_jkh_mo_ri(case):
    _, g, p = case
    a, b, c = orc.jkh_mo_ri(g["C"], g["H"], g["b"], p.nbf5)
    assert nrel(a, g["J_MO_ri"]) < TOL
    assert nrel(b, g["K_MO_ri"]) < TOL
    assert nrel(c, g["H_core"]) < TOL


def test_integrals_mo_ri(case):
    _, g, p = case
    Hmat, bmo = orc.integrals_mo_ri(g["C"], g["H"], g["b"], p.nbf5)
    assert nrel(Hmat, g["Hmat"]) < TOL
    assert nrel(bmo, g["b_MO"]) < TOL


def test_lagrange2_ri(case):
    _, g, p = case
    cj, ck = g["cj12"].copy(), g["ck12"].copy()
    elag, _ = orc.lagrange2(g["n_soft"], cj, ck, g["C"], g["H"], None, g["b"], p)
    assert nrel(elag, g["elag2_ri"]) < TOL
    assert np.all(np.diag(cj) == 0) and np.all(np.diag(ck) == 0)


def test_energy1r_routes(case):
    _, g, p = case
    E, elag, sd, md = orc.energy1r(g["C"], g["n_soft"], g["H"], None, g["b"], g["cj12"].copy(),
                                   g["ck12"].copy(), p)
    assert abs(E - float(g["E1r"])) < 1e-9 * max(1.0, abs(float(g["E1r"])))
    assert nrel(elag, g["elag1r"]) < TOL
    ph = types.SimpleNamespace(**vars(p))
    ph.no1 = p.nbeta
    nh = np.zeros(p.nbf5)
    nh[: p.nbeta] = 1.0
    Eh, elagh, _, _ = orc.energy1r(g["C"], nh, g["H"], None, g["b"], 2 * np.outer(nh, nh),
                                   np.outer(nh, nh), ph)
    assert abs(Eh - float(g["E1r_hf"])) < 1e-9 * max(1.0, abs(Eh))
    assert nrel(elagh, g["elag1r_hf"]) < TOL


def test_fock_route(case):
    _, g, p = case
    F = orc.fock_rc(g["J_ri"], g["K_ri"], g["n_soft"], g["H"], g["cj12"].copy(), g["ck12"].copy(), p)
    assert nrel(F, g["F_rc"]) < TOL
    elag = orc.lagrange(F, g["C"], p)
    assert nrel(elag, g["elag_F"]) < TOL
    E = orc.e_elec(g["H"], g["C"], g["n_soft"], elag, p)
    assert abs(E - float(g["E_F"])) < 1e-9 * max(1.0, abs(E))


def test_calce_and_orbital_gradient(case):
    _, g, p = case
    E = orc.calce(g["n_soft"], g["cj12"].copy(), g["ck12"].copy(), g["J_MO_ri"], g["K_MO_ri"],
                  g["H_core"], p)
    assert abs(E - float(g["E_calce"])) < 1e-10 * max(1.0, abs(E))
    elag, _ = orc.lagrange2(g["n_soft"], g["cj12"].copy(), g["ck12"].copy(), g["C"], g["H"], None,
                            g["b"], p)
    assert nrel(orc.orbital_gradient(elag, p), g["g_orb"]) < TOL
    assert nrel(orc.rotate_orbital(g["y"], g["C"], p), g["C_rot"]) < TOL


@pytest.mark.parametrize("name", ["c1", "water"])
def test_full_eri(name):
    g = load_golden(name)
    p = param_for(name)
    I = orc.eri_from_b(g["b"])
    J, K = orc.jkj_full(g["C"], I, p.nbf5)
    assert nrel(J, g["J_full"]) < TOL and nrel(K, g["K_full"]) < TOL
    a, b, _ = orc.jkh_mo_full(g["C"], g["H"], I, p.nbf5)
    assert nrel(a, g["J_MO_full"]) < TOL and nrel(b, g["K_MO_full"]) < TOL
    p.RI = False
    elag, _ = orc.lagrange2(g["n_soft"], g["cj12"].copy(), g["ck12"].copy(), g["C"], g["H"], I, None, p)
    assert nrel(elag, g["elag2_full"]) < TOL


@pytest.mark.parametrize("name", ["c1", "water"])
def test_hf_jk_helpers(name):
    """computeD_HF / computeDalpha_HF and their J, K (integrals.py:490-562);
    the alpha goldens follow JKalpha_HF_Full_GPU (the einsum route)."""
    g = load_golden(name)
    p = param_for(name)
    I = orc.eri_from_b(g["b"])
    D = orc.density_hf(g["C"], 0, p.nbeta)
    assert nrel(D, g["D_hf"]) < TOL
    J, K = orc.jk_hf_full(D, I)
    assert nrel(J, g["J_hf"]) < TOL and nrel(K, g["K_hf"]) < TOL
    Da = orc.density_hf(g["C"], p.nbeta, p.nbeta + 2)
    assert nrel(Da, g["Da_hf"]) < TOL
    Ja, Ka = orc.jk_hf_full(Da, I)
    assert nrel(Ja, g["Ja_hf"]) < TOL and nrel(Ka, g["Ka_hf"]) < TOL


@pytest.mark.parametrize("name", ["c1", "water"])
def test_post_nof_transforms(name):
    """compute_iajb / compute_pqrt (integrals.py:601-662)."""
    g = load_golden(name)
    p = param_for(name)
    I = orc.eri_from_b(g["b"])
    occ, vir, full = (p.no1, p.nalpha), (p.nalpha, p.nbf), (0, p.nbf)
    assert nrel(orc.mo4_full(g["C"], I, occ, vir, occ, vir), g["iajb"]) < TOL
    assert nrel(orc.mo4_full(g["C"], I, full, full, full, full), g["pqrt"]) < TOL


def open_shell_param(**over):
    from pynof_gb300 import synthetic

    with open(os.path.join(GOLDEN, "golden_meta.json")) as f:
        sizes = json.load(f)["open_shell"]["sizes"]
    st = synthetic.Structure(**sizes)
    for k, v in over.items():
        setattr(st, k, v)
    return st


def test_open_shell_fock_route():
    """computeF_RO_CPU (utils.py:97-169), computeLagrange, computeE_elec with
    both HighSpin settings, and ENERGY1r's no1 > 0, MSpin != 0 route; the
    in-place zeroing of the cj12 / ck12 diagonals from no1 on."""
    g = load_golden("open_shell")
    p = open_shell_param()
    cj, ck = g["cj12"].copy(), g["ck12"].copy()
    F = orc.fock_ro(g["J_ri"], g["K_ri"], g["n"], g["H"], cj, ck, p)
    assert nrel(F, g["F_ro"]) < TOL
    assert np.array_equal(cj, g["cj12_zeroed"]) and np.array_equal(ck, g["ck12_zeroed"])
    elag = orc.lagrange(F, g["C"], p)
    assert nrel(elag, g["elag_F"]) < TOL
    assert abs(orc.e_elec(g["H"], g["C"], g["n"], elag, p) - float(g["E_F"])) < TOL * abs(float(g["E_F"]))
    ph = open_shell_param(HighSpin=True)
    Eh = orc.e_elec(g["H"], g["C"], g["n"], elag, ph)
    assert abs(Eh - float(g["E_F_highspin"])) < TOL * abs(Eh)
    E, el1, sd, md = orc.energy1r(g["C"], g["n"], g["H"], None, g["b"], g["cj12"].copy(), g["ck12"].copy(), p)
    assert abs(E - float(g["E1r"])) < TOL * abs(E)
    assert nrel(el1, g["elag1r"]) < TOL


@pytest.mark.parametrize("case", ["c1", "water", "ragged"])
def test_occupations_coefficients_and_occupation_energy(case):
    """The oracle's softmax occupations, CJCKD8 and calcocce against the
    reference's own values (pnof.py:350-422, 770-809, 994-1001)."""
    from oracle import pynof_oracle as orc

    g = load_golden(case)
    p = param_for(case)
    n = orc.ocupacion_softmax(g["gamma"], p)
    assert np.max(np.abs(n - g["n_soft"])) < 1e-15
    cj, ck = orc.cjckd8(g["n_soft"], p)
    assert np.max(np.abs(cj - g["cj12"])) < 1e-15 and np.max(np.abs(ck - g["ck12"])) < 1e-15
    E = orc.calcocce(g["gamma"], g["J_MO_ri"], g["K_MO_ri"], g["H_core"], p)
    assert abs(E - float(g["E_calcocce"])) < 1e-12 * abs(E)
