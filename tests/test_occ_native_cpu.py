"""The library's compiled occupation function (gb_occ_energy_grad_f64, host
only) against nof.calcocce / nof.calcoccg, the restatements of
pnof.py:994-1033 tested against the oracle and finite differences.

Tolerances: E to 1e-13 relative; the gradient to 1e-12 of max(1, |g|_max)
(with saturated logits the whole gradient underflows towards 1e-60, where
only an absolute bound means anything)."""
import numpy as np
import pytest
import scipy.optimize

from pynof_gb300 import nof
from pynof_gb300.synthetic import Structure


@pytest.fixture(scope="module", autouse=True)
def built():
    from pynof_gb300 import _lib, build

    build.build()
    _lib.load()


STRUCTS = [dict(nbf=24, nbfaux=116, ndoc=4, ncwo=5), dict(nbf=24, nbfaux=116, ndoc=5, ncwo=3),
           dict(nbf=40, nbfaux=100, ndoc=4, ncwo=4, no1=2), dict(nbf=160, nbfaux=640, ndoc=16, ncwo=4),
           dict(nbf=60, nbfaux=100, ndoc=3, ncwo=1)]


def _mo(P, rng, asym):
    A = rng.standard_normal((P, P))
    B = rng.standard_normal((P, P))
    J = A @ A.T / P + asym * rng.standard_normal((P, P))
    K = B @ B.T / P + asym * rng.standard_normal((P, P))
    return J, K, rng.standard_normal(P)


@pytest.mark.parametrize("kw", STRUCTS, ids=lambda kw: "-".join(f"{k}{v}" for k, v in kw.items()))
@pytest.mark.parametrize("asym", [0.0, 0.01])
def test_native_matches_reference_formulas(kw, asym):
    st = Structure(**kw)
    rng = np.random.default_rng(st.nbf5 + int(asym * 1000))
    J, K, H = _mo(st.nbf5, rng, asym)
    f = nof.OccFunction(J, K, H, st)
    for scale in (0.3, 3.0, 400.0):
        gamma = rng.standard_normal(st.nv) * scale
        if scale > 100:
            gamma[0] = 800.0  # exp's range exceeded: the shifted softmax
        E, g = f(gamma)
        E0 = nof.calcocce(gamma, J, K, H, st)
        g0 = nof.calcoccg(gamma, J, K, H, st)
        assert abs(E - E0) <= 1e-13 * max(1.0, abs(E0))
        assert np.abs(g - g0).max() <= 1e-12 * max(1.0, np.abs(g0).max())


@pytest.mark.parametrize("name", ["c1", "water", "ragged"])
def test_native_cg_reaches_the_same_minimum(name):
    """scipy's CG (the reference's occupation optimiser) on the compiled
    function ends where it ends on the numpy one, on the MO integrals of the
    synthetic workloads (FP64, from the oracle)."""
    from oracle import pynof_oracle as orc
    from pynof_gb300 import synthetic

    st = synthetic.structure(name)
    b, C, Hao, _ = synthetic.make_inputs(st, 0)
    J, K, H = orc.jkh_mo_ri(C, Hao, b, st.nbf5)
    gamma0 = nof.gamma_guess_softmax(st)
    a = scipy.optimize.minimize(nof.OccFunction(J, K, H, st), gamma0, jac=True, method="CG")
    b = scipy.optimize.minimize(nof.calcocce, gamma0, args=(J, K, H, st), jac=nof.calcoccg, method="CG")
    assert abs(a.fun - b.fun) < 1e-10 * max(1.0, abs(b.fun))


def test_native_rejects_bad_layout():
    from pynof_gb300 import _lib

    J = np.eye(4)
    out = np.zeros(1)
    with pytest.raises(_lib.GBError):
        _lib.call("gb_occ_energy_grad_f64", np.zeros(8).ctypes.data, J.ctypes.data, J.ctypes.data,
                  np.zeros(4).ctypes.data, 4, 0, 2, 4, out.ctypes.data, None)


def test_calce_sums_with_compensation():
    """The energy sum keeps what plain FP64 summation loses: J_MO's large
    entries cancel in pairs (J_ji = -J_ij at 2^40), so E is the sum of the
    small dyadic parts alone (every product here is exact, so math.fsum of the
    terms is the exact E)."""
    import math
    import types

    P = 40
    rng = np.random.default_rng(11)
    i, j = np.indices((P, P))
    big = np.triu(rng.choice([-1.0, 1.0], size=(P, P)), 1) * 2.0 ** 40 * ((i + j) % 2 == 0)
    small = rng.integers(-2 ** 20, 2 ** 20, size=(P, P)) * 2.0 ** -40 * ((i + j) % 2 == 1)
    J = big - big.T + small  # large entries on one checkerboard colour, small ones on the other
    cj = np.ones((P, P))
    ck = np.zeros((P, P))
    p = types.SimpleNamespace(nbf5=P, nbeta=P // 2, nalpha=P // 2)
    n = np.zeros(P)
    E = nof.calce(n, cj.copy(), ck.copy(), J, np.zeros((P, P)), np.zeros(P), p)
    np.fill_diagonal(cj, 0.0)
    exact = math.fsum((cj * J.T).ravel())
    plain = float(np.sum(cj * J.T))
    print(f"exact {exact:.17g}  compensated {E:.17g}  plain {plain:.17g}")
    assert abs(E - exact) < 1e-10
