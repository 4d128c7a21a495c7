"""The CG restatement in oracle/occ_cg.py against scipy itself.

The reference minimises the occupation energy with scipy's CG
(``pynof/minimization.py:77-97``).  The restatement (Polak-Ribiere+ and the
More-Thuente line search, the device optimiser's checker) must take the same
steps: on the golden occupation problems and a synthetic one it reproduces
scipy's iterates bit for bit, with the same number of iterations and
function evaluations, where scipy's first line search always succeeds (its
fallback search is counted and must not run).
"""
import numpy as np
import pytest

from conftest import load_golden, param_for

scipy_opt = pytest.importorskip("scipy.optimize")


def _problems():
    for name in ("c1", "water", "ragged"):
        g = load_golden(name)
        yield name, param_for(name), g["gamma"], g["J_MO_ri"], g["K_MO_ri"], g["H_core"]
    from oracle import pynof_oracle as orc
    from pynof_gb300 import nof, synthetic

    st = synthetic.Structure.for_nbf(60)
    b, C, H, _ = synthetic.make_inputs(st, seed=1)
    J, K, Hc = orc.jkh_mo_ri(C, H, b, st.nbf5)
    yield "syn60", st, nof.gamma_guess_softmax(st), J, K, Hc


@pytest.mark.parametrize("case", ["c1", "water", "ragged", "syn60"])
def test_cg_restatement_matches_scipy(case, monkeypatch):
    import scipy.optimize._optimize as so

    from oracle import occ_cg
    from pynof_gb300 import nof

    name, p, g0, J, K, Hc = next(x for x in _problems() if x[0] == case)
    calls = {"fallback": 0}
    orig = so.line_search_wolfe2

    def counted(*a, **k):
        calls["fallback"] += 1
        return orig(*a, **k)

    monkeypatch.setattr(so, "line_search_wolfe2", counted)
    fn = nof.OccFunction(J, K, Hc, p)
    ref = scipy_opt.minimize(fn, g0, jac=True, method="CG")
    x, f, k, nev, ok = occ_cg.minimize_cg(fn, g0)
    assert calls["fallback"] == 0
    assert ok and ref.success
    assert k == ref.nit and nev == ref.nfev
    assert np.array_equal(x, ref.x)
    assert f == ref.fun


def test_cg_restatement_line_search_pieces():
    """The reverse-communication search on a 1-D quadratic: the first trial
    step of 1 on phi(a) = (a - 0.3)^2 brackets the minimum and the safeguarded
    steps converge to a point meeting the strong Wolfe conditions."""
    from oracle import occ_cg

    def phi(a):
        return (a - 0.3) ** 2, 2.0 * (a - 0.3)

    ls = occ_cg.LineSearch()
    f0, g0 = phi(0.0)
    task, stp = ls.start(1.0, f0, g0)
    n = 0
    while task == "FG":
        f, g = phi(stp)
        task, stp = ls.step(f, g)
        n += 1
    assert task == "CONV" and n < 10
    f, g = phi(stp)
    assert f <= f0 + 1e-4 * stp * g0 and abs(g) <= 0.4 * abs(g0)
    # an ascent direction fails at once, as scipy's search does
    assert occ_cg.LineSearch().start(1.0, 0.0, 1.0) == ("FAIL", None)
