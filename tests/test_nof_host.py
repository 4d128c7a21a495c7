"""Host occupation / orbital math against the reference's outputs (golden)."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, nrel, param_for
from pynof_gb300 import nof

TOL = 1e-12


@pytest.fixture(params=sorted(GOLDEN_CASES))
def case(request):
    name = request.param
    return load_golden(name), param_for(GOLDEN_CASES[name])


def test_softmax_occupations(case):
    g, p = case
    n, dn = nof.ocupacion_softmax(g["gamma"], p)
    assert nrel(n, g["n_soft"]) < TOL
    assert nrel(dn, g["dn_soft"]) < TOL


def test_gnof_coefficients_and_derivatives(case):
    g, p = case
    cj, ck = nof.cjckd8(g["n_soft"], p)
    assert nrel(cj, g["cj12"]) < TOL and nrel(ck, g["ck12"]) < TOL
    Dcj, Dck = nof.der_cjckd8(g["n_soft"], g["dn_soft"], p)
    assert nrel(Dcj, g["Dcj12"]) < TOL and nrel(Dck, g["Dck12"]) < TOL


def test_occupation_energy_and_gradient(case):
    g, p = case
    E = nof.calce(g["n_soft"], g["cj12"].copy(), g["ck12"].copy(), g["J_MO_ri"], g["K_MO_ri"], g["H_core"], p)
    assert abs(E - float(g["E_calce"])) < 1e-11 * abs(E)
    Eo = nof.calcocce(g["gamma"], g["J_MO_ri"], g["K_MO_ri"], g["H_core"], p)
    assert abs(Eo - float(g["E_calcocce"])) < 1e-11 * abs(Eo)
    go = nof.calcoccg(g["gamma"], g["J_MO_ri"], g["K_MO_ri"], g["H_core"], p)
    assert nrel(go, g["g_occ"]) < 1e-11


def test_occupation_gradient_finite_difference(case):
    """calcoccg against central differences of calcocce (the pair the
    reference writes side by side, pnof.py:994-1033)."""
    g, p = case
    gam = g["gamma"]
    ga = nof.calcoccg(gam, g["J_MO_ri"], g["K_MO_ri"], g["H_core"], p)
    h = 1e-6
    fd = np.zeros_like(gam)
    for k in range(len(gam)):
        e = np.zeros_like(gam)
        e[k] = h
        fd[k] = (nof.calcocce(gam + e, g["J_MO_ri"], g["K_MO_ri"], g["H_core"], p)
                 - nof.calcocce(gam - e, g["J_MO_ri"], g["K_MO_ri"], g["H_core"], p)) / (2 * h)
    assert nrel(ga, fd) < 1e-6


def test_orbital_gradient_rotation_ordering(case):
    g, p = case
    assert nrel(nof.orbital_gradient(g["elag2_ri"], p), g["g_orb"]) < TOL
    assert nrel(nof.rotate_orbital(g["y"], g["C"], p), g["C_rot"]) < TOL
    Cs, gs = nof.order_occupations_softmax(g["C"], g["gamma"], p)
    assert nrel(Cs, g["C_sorted"]) < TOL
    assert np.allclose(gs, g["gamma_sorted"], rtol=0, atol=1e-14)


@pytest.mark.parametrize("nbf,ncwo,no1", [(24, 4, 0), (37, 3, 0), (60, 2, 0), (160, 4, 0), (40, 3, 2)])
def test_calcoccg_fast_equals_dense(nbf, ncwo, no1):
    """The contraction form of the occupation gradient equals calcoccg (the
    dense restatement of pnof.py:1004-1033) on random J_MO, K_MO, H_core."""
    from pynof_gb300 import nof, synthetic

    st = synthetic.Structure(nbf=nbf, nbfaux=4 * nbf, ndoc=max(1, nbf // 10), ncwo=ncwo, no1=no1)
    P = st.nbf5
    rng = np.random.default_rng(nbf + ncwo)
    A = rng.standard_normal((P, P))
    J = A @ A.T / P + 0.01 * rng.standard_normal((P, P))
    B = rng.standard_normal((P, P))
    K = B @ B.T / P
    Hc = rng.standard_normal(P)
    g = nof.gamma_guess_softmax(st) + 0.5 * rng.standard_normal(st.nv)
    a = nof.calcoccg(g, J, K, Hc, st)
    b = nof.calcoccg_fast(g, J, K, Hc, st)
    assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()
