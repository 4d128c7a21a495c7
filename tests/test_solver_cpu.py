"""The solve loop's host logic (occoptr with the compiled occupation function,
orbopt_adam with the compensated calce, order_occupations_softmax, the
convergence test) against the reference's recorded water trajectory, on the
CPU: the device contractions are stood in for by the oracle.

Same checks as the device-backed test (tests/test_gpu_solver.py)."""
import numpy as np

from conftest import load_golden, nrel, param_for


class OracleBackend:
    """The Backend interface of pynof_gb300.solver with the oracle's FP64
    restatements in place of the device calls."""

    precision = "fp64"

    def __init__(self, p, b, H):
        from oracle import pynof_oracle as orc

        self.orc, self.p, self.b, self.H = orc, p, b, H
        self.C = self.best = None

    def jkh_mo(self, C):
        return self.orc.jkh_mo_ri(C, self.H, self.b, self.p.nbf5)

    def lagrange2(self, C, n, cj12, ck12):
        return self.orc.lagrange2(n, cj12.copy(), ck12.copy(), C, self.H, None, self.b, self.p)

    def rotate(self, y, C):
        return self.orc.rotate_orbital(y, C, self.p)

    def _at(self):
        J, K, Hc = self.jkh_mo(self.C)
        elag, _ = self.lagrange2(self.C, self.n, self.cj, self.ck)
        return J, K, Hc, elag

    def orbital_begin(self, C, n, cj12, ck12):
        self.C, self.n, self.cj, self.ck = C.copy(), n.copy(), cj12.copy(), ck12.copy()
        self.best = self.C.copy()
        return self._at()

    def orbital_step(self, y):
        self.C = self.rotate(y, self.C)
        return self._at()

    def keep_best(self):
        self.best = self.C.copy()

    def best_C(self):
        return self.best.copy()

    def set_precision(self, *args, **kwargs):
        pass


def test_host_loop_matches_reference_trajectory():
    from pynof_gb300 import build, solver

    build.build()  # the compiled occupation function and calce live in the library
    g = load_golden("loop_water")
    p = param_for("water")
    res = solver.solve(OracleBackend(p, g["b"], g["H"]), g["C0"].copy(), g["gamma0"].copy(), p, tol=0.0,
                       maxit=len(g["E_orb"]))
    h = res.history
    assert np.allclose(h["E_orb"], g["E_orb"], rtol=1e-9, atol=0)
    assert np.allclose(h["E_occ"], g["E_occ"], rtol=1e-9, atol=0)
    assert np.allclose(h["g_orb"], g["g_orb"], rtol=1e-7, atol=0)
    assert np.allclose(h["g_occ"], g["g_occ"], rtol=1e-5, atol=0)
    last = len(g["E_orb"]) - 1
    assert nrel(res.C, g[f"C_{last}"]) < 1e-6
    assert nrel(res.gamma, g[f"gamma_{last}"]) < 1e-6
