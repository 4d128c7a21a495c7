"""The occupation optimiser on the device (gb_occ_minimize_dev,
gb_occ_energy_grad_dev) against the host evaluation and scipy's CG.

* one evaluation E(gamma), dE/dgamma against the compiled host loop
  (gb_occ_energy_grad_f64, itself pinned to the reference's calcocce /
  calcoccg golden values) on the golden problems, a synthetic one from the
  oracle's J_MO / K_MO, an nbf5 = 300 problem, inactive core orbitals
  (no1 > 0), one weak orbital per pair, and logits past exp's range;
* the whole minimisation against scipy's CG on the host (the reference's
  optimiser, ``pynof/minimization.py:77-97``): same minimum (energy to
  1e-12 relative, gamma to 1e-6), converged to gtol;
* the step sequence against the CPU restatement of scipy's CG
  (oracle/occ_cg.py) driven by the device's own evaluations: the same
  iterations and evaluations;
* the occupations and C^J, C^K written at the result against
  ocupacion_softmax / CJCKD8 at the returned gamma;
* edge cases: maxiter = 0, a non-finite H_core (the loop ends, no success),
  gamma_out aliasing gamma0, one object reused for two problems.
"""
import numpy as np
import pytest

from conftest import load_golden, nrel, param_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _problem(case):
    from pynof_gb300 import nof, synthetic

    if case in ("c1", "water", "ragged"):
        g = load_golden(case)
        return param_for(case), g["gamma"], g["J_MO_ri"], g["K_MO_ri"], g["H_core"]
    if case == "syn120":
        from oracle import pynof_oracle as orc

        st = synthetic.Structure.for_nbf(120)
        b, C, H, _ = synthetic.make_inputs(st, seed=1)
        J, K, Hc = orc.jkh_mo_ri(C, H, b, st.nbf5)
        return st, nof.gamma_guess_softmax(st), J, K, Hc
    if case in ("no1", "ncwo1"):
        # inactive core orbitals (no1 > 0), or one weak orbital per pair
        st = synthetic.Structure(nbf=40, nbfaux=160, ndoc=4, ncwo=3, no1=2) if case == "no1" else \
            synthetic.Structure(nbf=40, nbfaux=160, ndoc=6, ncwo=1)
    else:
        # nbf5 = 300 (the nbf=600 structure)
        st = synthetic.structure("c3")
    # symmetric positive J, K with a dominant diagonal, H_core spread over
    # the orbitals
    P = st.nbf5
    rng = np.random.default_rng(5)
    A = 0.01 * rng.standard_normal((P, P))
    B = 0.01 * rng.standard_normal((P, P))
    J = np.abs(A + A.T) + np.eye(P)
    K = np.abs(B + B.T) + np.eye(P)
    Hc = -np.linspace(5.0, 0.1, P)
    return st, nof.gamma_guess_softmax(st), J, K, Hc


def _dev(*xs):
    from pynof_gb300 import ops

    return [ops.to_device(np.ascontiguousarray(x, dtype=np.float64)) for x in xs]


CASES = ["c1", "water", "ragged", "syn120", "p300", "no1", "ncwo1"]


@pytest.mark.parametrize("case", CASES)
def test_energy_grad_matches_host(torch_cuda, case):
    from pynof_gb300 import nof, ops

    p, g0, J, K, Hc = _problem(case)
    fn = nof.OccFunction(J, K, Hc, p)
    om = ops.OccMinimizer(p.nbf5, p.no1, p.ndoc, p.ncwo)
    dJ, dK, dH = _dev(J, K, Hc)
    rng = np.random.default_rng(3)
    points = [g0, g0 + 0.3 * rng.standard_normal(g0.size)]
    big = g0.copy()
    big[:: max(1, big.size // 3)] = 705.0  # the shifted softmax
    points.append(big)
    for x in points:
        E, g = fn(x)
        res, grad = om.energy_grad(*_dev(x), dJ, dK, dH)
        r = res.cpu().numpy()
        gd = grad.cpu().numpy()
        assert abs(r[0] - E) <= 1e-13 * abs(E), (case, r[0], E)
        assert nrel(gd, g) < 1e-11, (case, nrel(gd, g))
        assert r[4] == np.max(np.abs(gd))


@pytest.mark.parametrize("case", CASES)
def test_minimize_matches_scipy(torch_cuda, case):
    import scipy.optimize

    from pynof_gb300 import nof, ops

    p, g0, J, K, Hc = _problem(case)
    fn = nof.OccFunction(J, K, Hc, p)
    ref = scipy.optimize.minimize(fn, g0, jac=True, method="CG")
    om = ops.OccMinimizer(p.nbf5, p.no1, p.ndoc, p.ncwo)
    gam, res = om.minimize(*_dev(g0, J, K, Hc), coefficients=False)[:2]
    r = res.cpu().numpy()
    x = gam.cpu().numpy()
    print(f"{case}: device E {r[0]:.15e} nit {r[1]:.0f} nev {r[2]:.0f} ok {r[3]:.0f} |g| {r[4]:.2e}; "
          f"scipy E {ref.fun:.15e} nit {ref.nit} nfev {ref.nfev}")
    assert r[3] == 1.0 and r[4] <= 1e-5
    assert abs(r[0] - ref.fun) <= 1e-12 * abs(ref.fun)
    assert nrel(x, ref.x) < 1e-6
    # the returned energy is the one at the returned gamma
    assert abs(fn.energy(x) - r[0]) <= 1e-13 * abs(r[0])


@pytest.mark.parametrize("case", ["c1", "ragged", "syn120"])
def test_minimize_follows_restatement(torch_cuda, case):
    """The restatement of scipy's CG, fed the device's own evaluations, takes
    the same number of iterations and evaluations as the device loop."""
    from oracle import occ_cg
    from pynof_gb300 import ops

    p, g0, J, K, Hc = _problem(case)
    dJ, dK, dH = _dev(J, K, Hc)
    ev = ops.OccMinimizer(p.nbf5, p.no1, p.ndoc, p.ncwo)

    def fg(x):
        res, grad = ev.energy_grad(*_dev(x), dJ, dK, dH)
        return float(res[0].item()), grad.cpu().numpy().copy()

    x, f, k, nev, ok = occ_cg.minimize_cg(fg, g0)
    om = ops.OccMinimizer(p.nbf5, p.no1, p.ndoc, p.ncwo)
    r = om.minimize(*_dev(g0), dJ, dK, dH, coefficients=False)[1].cpu().numpy()
    print(f"{case}: device nit {r[1]:.0f} nev {r[2]:.0f}; restatement nit {k} nev {nev}")
    assert ok and r[3] == 1.0
    assert (int(r[1]), int(r[2])) == (k, nev)
    assert abs(r[0] - f) <= 1e-13 * abs(f)


@pytest.mark.parametrize("case", ["c1", "syn120"])
def test_minimize_writes_occupations_and_coefficients(torch_cuda, case):
    from pynof_gb300 import nof, ops

    p, g0, J, K, Hc = _problem(case)
    om = ops.OccMinimizer(p.nbf5, p.no1, p.ndoc, p.ncwo)
    gam, res, n, cj, ck = om.minimize(*_dev(g0, J, K, Hc))
    x = gam.cpu().numpy()
    n_ref, _ = nof.ocupacion_softmax(x, p)
    nd = n.cpu().numpy()
    assert nrel(nd, n_ref) < 1e-14
    cj_ref, ck_ref = nof.cjckd8(nd, p)
    assert nrel(cj.cpu().numpy(), cj_ref) < 1e-14
    assert nrel(ck.cpu().numpy(), ck_ref) < 1e-14


def test_minimize_edge_cases(torch_cuda):
    from pynof_gb300 import nof, ops

    p, g0, J, K, Hc = _problem("water")
    fn = nof.OccFunction(J, K, Hc, p)
    dJ, dK, dH = _dev(J, K, Hc)
    om = ops.OccMinimizer(p.nbf5, p.no1, p.ndoc, p.ncwo)
    # no iterations: the energy at gamma0, gamma unchanged
    gam, res = om.minimize(*_dev(g0), dJ, dK, dH, maxiter=0, coefficients=False)[:2]
    r = res.cpu().numpy()
    assert r[1] == 0 and r[2] == 1 and abs(r[0] - fn.energy(g0)) <= 1e-13 * abs(r[0])
    assert np.array_equal(gam.cpu().numpy(), g0)
    # gamma_out aliasing gamma0, then a second problem on the same object
    om.gamma.copy_(_dev(g0)[0])
    r1 = om.minimize(om.gamma, dJ, dK, dH, coefficients=False)[1].cpu().numpy().copy()
    p2, g2, J2, K2, H2 = _problem("c1")
    om2 = ops.OccMinimizer(p2.nbf5, p2.no1, p2.ndoc, p2.ncwo)
    r2 = om2.minimize(*_dev(g2, J2, K2, H2), coefficients=False)[1].cpu().numpy()
    r1b = om.minimize(*_dev(g0), dJ, dK, dH, coefficients=False)[1].cpu().numpy()
    assert r1[3] == 1.0 and r2[3] == 1.0 and np.array_equal(r1, r1b)
    # a non-finite input: the loop ends at once without success
    Hbad = Hc.copy()
    Hbad[0] = np.nan
    r = om.minimize(*_dev(g0), dJ, dK, *_dev(Hbad), coefficients=False)[1].cpu().numpy()
    assert r[3] == 0.0 and r[2] == 1
    om.close()
    om2.close()


@pytest.mark.parametrize("case", ["water", "ragged"])
def test_dropin_occoptr(torch_cuda, case):
    """``minimization.occoptr`` (what the installer binds to ``pynof.occoptr``)
    against the reference's occoptr restated on the host: the oracle's J_MO,
    K_MO, H_core, scipy's CG over calcocce / calcoccg, then the occupations
    and CJCKD8 at the result (minimization.py:77-97)."""
    import scipy.optimize

    from oracle import pynof_oracle as orc
    from pynof_gb300 import minimization, nof, ops

    g = load_golden(case)
    p = param_for(case)
    J, K, Hc = orc.jkh_mo_ri(g["C"], g["H"], g["b"], p.nbf5)
    ref = scipy.optimize.minimize(nof.calcocce, g["gamma"], args=(J, K, Hc, p), jac=nof.calcoccg, method="CG")
    E, nit, ok, gam, n, cj, ck = minimization.occoptr(g["gamma"], g["C"], g["H"], None, ops.to_device(g["b"]), p)
    assert ok and ref.success and nit > 0
    assert abs(E - ref.fun) <= 1e-10 * abs(ref.fun)
    assert nrel(gam, ref.x) < 1e-5
    n_ref, _ = nof.ocupacion_softmax(ref.x, p)
    cj_ref, ck_ref = nof.cjckd8(n_ref, p)
    assert nrel(n, n_ref) < 1e-6 and nrel(cj, cj_ref) < 1e-6 and nrel(ck, ck_ref) < 1e-6


@pytest.mark.parametrize("case", ["c1", "syn120", "p300"])
def test_host_driven_matches_graph(torch_cuda, case):
    """gb_occ_minimize_dev_sync (replays of an ordinary graph, the phase read
    back after each) runs the same kernels and steps as the conditional-node
    graph: bit-identical gamma, result, n, C^J, C^K."""
    from pynof_gb300 import ops

    p, g0, J, K, Hc = _problem(case)
    dg, dJ, dK, dH = _dev(g0, J, K, Hc)
    om = ops.OccMinimizer(p.nbf5, p.no1, p.ndoc, p.ncwo)
    a = [t.cpu().numpy().copy() for t in om.minimize(dg, dJ, dK, dH)]
    b = [t.cpu().numpy().copy() for t in om.minimize(dg, dJ, dK, dH, host_driven=True)]
    assert b[1][3] == 1.0
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
