"""psi4-free NOF solve loop over the device kernels.

Restates the orbital / occupation optimisation of ``pynof.compute_energy``
(``energy.py:94-170``) -- ``occoptr`` (``minimization.py:77-97``, scipy CG
over the softmax gammas), ``orbopt_adam`` (``minimization.py:200-253``,
AMSgrad on orbital rotations), ``order_occupations_softmax``
(``guess.py:77-106``) and the convergence test on the two gradient norms --
with every four-index contraction (``computeJKH_MO``, ``computeLagrange2``),
the orbital rotation (``rotate_orbital``, FP64 expm) and, by default, the
occupation optimiser (scipy's CG over calcocce / calcoccg as one device graph,
:class:`ops.OccMinimizer`) on the GPU; the AMSgrad bookkeeping and the
remaining occupation-space math run in FP64 on the host
(:mod:`pynof_gb300.nof`).

A :class:`Backend` owns one molecule's resident device state (b, its sliced
form for the tensor-core path, H) and a CUDA stream, so several solves can
run concurrently (the serving loop).
"""
from __future__ import annotations

import copy
import dataclasses
import time

import numpy as np
import scipy.optimize
import torch

from . import integrals, nof, ops


class Backend:
    """Device contractions for one molecule.

    precision: "fp64" (DMMA) or "mixed" (tcgen05 digit slices, ``nslices``).

    The orbital steps of the AMSgrad loop keep C resident on the device
    (``orbital_begin`` / ``orbital_step`` / ``keep_best`` / ``best_C``).  With
    ``use_graphs`` each step -- rotation C expm(Y), computeJKH_MO and
    computeLagrange2 at the new orbitals -- is one CUDA-graph replay, captured
    once per (precision, number of expm squarings)."""

    def __init__(self, st, b, H, precision: str = "mixed", nslices: int = 6, device=None, stream=None,
                 use_graphs: bool = True, occupations: str = "device"):
        if occupations not in ("device", "device_sync", "host"):
            raise ValueError(f"occupations must be 'device', 'device_sync' or 'host', got {occupations!r}")
        self.st = st
        self.use_graphs = use_graphs
        # "device": occoptr's CG runs on the device (ops.OccMinimizer, one
        # conditional-node graph) at the device J_MO, K_MO, H_core;
        # "device_sync": the same kernels driven from the host in replays of
        # eight evaluations; "host": scipy's CG over the compiled host
        # evaluation (scipy's own iterates)
        self.occupations = occupations
        self._occ = None
        self._norm = ops.AntisymNorm(st.nbf, st.nbf5)
        self._graphs: dict = {}
        self._buf: dict | None = None
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.stream = stream if stream is not None else torch.cuda.Stream(self.device)
        self.precision = precision
        self.nslices = nslices
        with torch.cuda.stream(self.stream):
            self.b = ops.to_device(b, self.device)
            self.H = ops.to_device(H, self.device)
            self.prep = ops.PreparedRI(self.b, nslices) if precision == "mixed" else None
        self.calls = {"jkh_mo": 0, "lagrange2": 0}

    def set_precision(self, precision: str, nslices: int | None = None):
        """Switch arithmetic (e.g. to FP64 near convergence)."""
        self.precision = precision
        self._graphs.clear()  # the new path may need a larger workspace: recapture
        if nslices is not None and nslices != self.nslices:
            self.nslices = nslices
            self.prep = None
        if precision == "mixed" and self.prep is None:
            with torch.cuda.stream(self.stream):
                self.prep = ops.PreparedRI(self.b, self.nslices)

    def nbytes(self) -> int:
        n = self.b.numel() * 8 + self.H.numel() * 8
        if self.prep is not None:
            n += self.prep.buf.numel()
        return n

    def _sync_host(self, *ts):
        with torch.cuda.stream(self.stream):
            out = [t.to("cpu", non_blocking=False) for t in ts]
        # after this stream's work: a timed-out or non-finite split-product
        # call raises here instead of feeding unwritten results to the loop
        ops.check_device_status()
        return [o.numpy() for o in out]

    # device-side pieces (current stream = self.stream)
    def _jkh_mo_dev(self, dC):
        self.calls["jkh_mo"] += 1
        if self.precision == "mixed":
            return ops.jkh_mo_ri_mixed(dC, self.H, self.prep, self.st.nbf5)
        return ops.jkh_mo_ri(dC, self.H, self.b, self.st.nbf5)

    def _lagrange2_dev(self, dC, dn, dcj, dck):
        self.calls["lagrange2"] += 1
        st = self.st
        if self.precision == "mixed":
            return ops.lagrange2_ri_mixed(dC, self.H, self.prep, dn, dcj, dck, st.nbf5, st.nbeta, st.nalpha)
        return ops.lagrange2_ri(dC, self.H, self.b, dn, dcj, dck, st.nbf5, st.nbeta, st.nalpha)

    def jkh_mo(self, C):
        with torch.cuda.stream(self.stream):
            return self._sync_host(*self._jkh_mo_dev(ops.to_device(C, self.device)))

    # ---- occupations on the device ----------------------------------------
    def _occ_min(self):
        if self._occ is None:
            st = self.st
            self._occ = ops.OccMinimizer(st.nbf5, st.no1, st.ndoc, st.ncwo, self.device)
        return self._occ

    def occ_minimize(self, gamma, C):
        """occoptr's CG at orbitals C on the device: J_MO, K_MO, H_core stay
        on the device; returns host (E, iterations, success, gamma, n, cj12,
        ck12) from one synchronisation."""
        with torch.cuda.stream(self.stream):
            J, K, Hc = self._jkh_mo_dev(ops.to_device(C, self.device))
            om = self._occ_min()
            gam, res, n, cj, ck = om.minimize(ops.to_device(gamma, self.device), J, K, Hc,
                                              host_driven=self.occupations == "device_sync")
            gam, res, n, cj, ck = self._sync_host(gam, res, n, cj, ck)
        if res[3] < 0:
            raise RuntimeError("occupation minimiser reached its evaluation cap")
        return float(res[0]), int(res[1]), bool(res[3] == 1.0), gam, n, cj, ck

    def occ_gradient(self, gamma, C):
        """dE/dgamma (calcoccg) at orbitals C, evaluated on the device."""
        with torch.cuda.stream(self.stream):
            J, K, Hc = self._jkh_mo_dev(ops.to_device(C, self.device))
            _, grad = self._occ_min().energy_grad(ops.to_device(gamma, self.device), J, K, Hc)
            return self._sync_host(grad)[0]

    # ---- device-resident orbital steps ---------------------------------
    def _static(self):
        if self._buf is None:
            N, P, nvar = self.st.nbf, self.st.nbf5, self.st.nvar

            def z(*shape):
                return torch.zeros(shape, dtype=torch.float64, device=self.device)

            self._buf = {"C": z(N, N), "Cprev": z(N, N), "best": z(N, N), "y": z(nvar), "n": z(P), "cj": z(P, P),
                         "ck": z(P, P), "J": z(P, P), "K": z(P, P), "Hc": z(P), "elag": z(N, N), "Hmat": z(N, P)}
        return self._buf

    def _step_body(self, sq):
        """Rotation by the static y with sq squarings (none when sq < 0), then
        the two contractions at the static C into the static outputs.  Issues
        launches only (no allocation, no synchronisation)."""
        b, st = self._static(), self.st
        if sq >= 0:
            b["Cprev"].copy_(b["C"])
            ops.rotate_orbital(b["y"], b["Cprev"], st.nbf5, out=b["C"], norm1=0.5 * 2.0 ** sq)
        self.calls["jkh_mo"] += 1
        self.calls["lagrange2"] += 1
        mo_out, l2_out = (b["J"], b["K"], b["Hc"]), (b["elag"], b["Hmat"])
        if self.precision == "mixed":
            # one call: the half transform and the MO transform serve both
            ops.jkh_lagrange2_ri_mixed(b["C"], self.H, self.prep, b["n"], b["cj"], b["ck"], st.nbf5, st.nbeta,
                                       st.nalpha, out=mo_out + l2_out)
        else:
            ops.jkh_mo_ri(b["C"], self.H, self.b, st.nbf5, out=mo_out)
            ops.lagrange2_ri(b["C"], self.H, self.b, b["n"], b["cj"], b["ck"], st.nbf5, st.nbeta, st.nalpha,
                             out=l2_out)

    def _run_step(self, sq):
        b = self._static()
        with torch.cuda.stream(self.stream):
            if not self.use_graphs:
                self._step_body(sq)
            else:
                key = (self.precision, self.nslices, sq)
                g = self._graphs.get(key)
                if g is None:
                    # grow the workspaces in a plain run on a copy of the state,
                    # then capture (thread-local mode: other requests' threads
                    # keep running)
                    saved = b["C"].clone()
                    self._step_body(sq)
                    b["C"].copy_(saved)
                    g = ops.StreamGraph(self.stream)
                    g.begin()
                    try:
                        self._step_body(sq)
                    finally:
                        g.end()
                    self._graphs[key] = g
                g.launch()
            return self._sync_host(b["J"], b["K"], b["Hc"], b["elag"])

    def orbital_begin(self, C, n, cj12, ck12):
        """Load C, n, cj12, ck12 (diagonals already zero) and return host
        (J_MO, K_MO, H_core, elag) at C."""
        b = self._static()
        with torch.cuda.stream(self.stream):
            for k, x in (("C", C), ("n", n), ("cj", cj12), ("ck", ck12)):
                b[k].copy_(torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)))
            b["best"].copy_(b["C"])
        return tuple(self._run_step(-1))

    def orbital_step(self, y):
        """C <- C expm(Y(y)) on the device; host (J_MO, K_MO, H_core, elag) at the new C."""
        b = self._static()
        nrm = self._norm(y)
        if not np.isfinite(nrm):
            raise FloatingPointError("orbital step is not finite")
        sq = 0
        while nrm > 0.5:
            nrm *= 0.5
            sq += 1
        with torch.cuda.stream(self.stream):
            b["y"].copy_(torch.from_numpy(np.ascontiguousarray(y, dtype=np.float64)))
        return tuple(self._run_step(sq))

    def keep_best(self):
        with torch.cuda.stream(self.stream):
            self._static()["best"].copy_(self._static()["C"])

    def best_C(self):
        return self._sync_host(self._static()["best"])[0]

    def lagrange2(self, C, n, cj12, ck12):
        with torch.cuda.stream(self.stream):
            dn, dcj, dck = (ops.to_device(x, self.device) for x in (n, cj12, ck12))
            return self._sync_host(*self._lagrange2_dev(ops.to_device(C, self.device), dn, dcj, dck))


@dataclasses.dataclass
class SolveState:
    """Optimizer settings the reference keeps on ``param`` and mutates
    (``minimization.py:248-250``)."""

    alpha: float = 0.02
    maxloop: int = 30


def calcorbe(y, n, cj12, ck12, C, be, p):
    """``pnof.py:1103-1111``."""
    Cn = C if not np.any(y) else be.rotate(y, C)
    J_MO, K_MO, H_core = be.jkh_mo(Cn)
    return nof.calce(n, cj12, ck12, J_MO, K_MO, H_core, p)


def calcorbg(y, n, cj12, ck12, C, be, p):
    """``pnof.py:1114-1131``."""
    Cn = C if not np.any(y) else be.rotate(y, C)
    np.fill_diagonal(cj12, 0.0)
    np.fill_diagonal(ck12, 0.0)
    elag, _ = be.lagrange2(Cn, n, cj12, ck12)
    return nof.orbital_gradient(elag, p)


def occoptr(gamma, C, be, p):
    """``minimization.py:77-97``: CG over gamma at fixed orbitals -- on the
    device when the backend's ``occupations`` is "device" (closed shell),
    else scipy's CG over the compiled host evaluation."""
    if p.ndoc > 0 and getattr(be, "occupations", "host") != "host" and nof.native_occ_ok(p):
        return be.occ_minimize(gamma, C)
    J_MO, K_MO, H_core = be.jkh_mo(C)
    E, nit, success = 0.0, 0, True
    if p.ndoc > 0:
        if nof.native_occ_ok(p):
            # the compiled E and dE/dgamma in one call (the same CG iterates)
            res = scipy.optimize.minimize(nof.OccFunction(J_MO, K_MO, H_core, p), gamma, jac=True, method="CG")
        else:
            res = scipy.optimize.minimize(nof.calcocce, gamma, args=(J_MO, K_MO, H_core, p),
                                          jac=nof.calcoccg_fast, method="CG")
        gamma, E, nit, success = res.x, res.fun, res.nit, res.success
    n, _ = nof.ocupacion_softmax(gamma, p)
    cj12, ck12 = nof.cjckd8(n, p)
    return E, nit, success, gamma, n, cj12, ck12


def orbopt_adam(gamma, C, be, p, state: SolveState, deadline: float | None = None):
    """``minimization.py:200-253``: AMSgrad steps of orbital rotations (no
    further steps once ``time.perf_counter()`` passes ``deadline``)."""
    n, _ = nof.ocupacion_softmax(gamma, p)
    cj12, ck12 = nof.cjckd8(n, p)
    np.fill_diagonal(cj12, 0.0)  # as calce / calcorbg do in place
    np.fill_diagonal(ck12, 0.0)
    # C stays on the device for the whole loop: E (calcorbe) and the gradient
    # (calcorbg) at the same orbitals come from one device round trip, and so
    # do the rotation plus both contractions after each step
    J_MO, K_MO, H_core, elag = be.orbital_begin(C, n, cj12, ck12)
    E = nof.calce(n, cj12, ck12, J_MO, K_MO, H_core, p)
    alpha, beta1, beta2 = state.alpha, 0.7, 0.999
    m = np.zeros(p.nvar)
    v = np.zeros(p.nvar)
    vhat_max = np.zeros(p.nvar)
    improved = success = False
    best_E, best_C = E, C
    nit = 0
    for i in range(state.maxloop):
        if deadline is not None and i > 0 and time.perf_counter() > deadline:
            break
        nit += 1
        grad = nof.orbital_gradient(elag, p)
        if np.linalg.norm(grad) < 1e-4 and improved:
            success = True
            break
        m = beta1 * m + (1 - beta1) * grad
        v = beta2 * v + (1 - beta2) * grad ** 2
        mhat = m / (1.0 - beta1 ** (i + 1))
        vhat = v / (1.0 - beta2 ** (i + 1))
        vhat_max = np.maximum(vhat_max, vhat)
        y = -alpha * mhat / np.sqrt(vhat_max + 1e-8)
        J_MO, K_MO, H_core, elag = be.orbital_step(y)
        E = nof.calce(n, cj12, ck12, J_MO, K_MO, H_core, p)
        if E < best_E:
            be.keep_best()
            best_E = E
            improved = True
    if improved:
        best_C = be.best_C()
    if not improved:
        state.alpha /= 10
        state.maxloop += 30
    return best_E, best_C, nit, success


@dataclasses.dataclass
class SolveResult:
    E_elec: float
    C: np.ndarray
    gamma: np.ndarray
    n: np.ndarray
    iterations: int
    converged: bool
    history: dict
    seconds: float


def solve(be: Backend, C, gamma, p, tol: float = 1e-3, maxit: int = 1000, fp64_switch: float | None = None,
          callback=None, ladder=None, final_fp64: bool = False, time_limit: float | None = None) -> SolveResult:
    """The outer loop of ``compute_energy`` (``energy.py:112-170``).

    Converged when both gradient norms are below ``tol`` (or their optimizers
    report success), as ``energy.py:155`` (whose tolerance is 1e-3).

    Precision is switched up as the orbital gradient norm falls: ``ladder``
    is a sequence of (threshold, precision, nslices) rungs taken in order,
    each once the norm is below its threshold (e.g. bf16x3 digits first, then
    six digits at 1e-2); ``fp64_switch`` is the one-rung ladder to the FP64
    path.  With ``final_fp64`` the closing Lagrangian (the reported energy) is
    evaluated on the FP64 path.  ``time_limit`` (seconds) ends the loop
    unconverged once it has passed (orbital steps stop at the limit, the outer
    iteration in progress completes)."""
    t0 = time.perf_counter()
    rungs = list(ladder or [])
    if fp64_switch is not None:
        rungs.append((fp64_switch, "fp64", None))
    p = copy.copy(p)
    state = SolveState(alpha=getattr(p, "alpha", 0.02), maxloop=getattr(p, "maxloop", 30))
    hist = {k: [] for k in ("E_orb", "E_occ", "g_orb", "g_occ", "nit_orb", "nit_occ", "precision")}
    # wall time of the occupation CG and of the orbital steps (seconds)
    hist["t_occ"] = 0.0
    hist["t_orb"] = 0.0
    t = time.perf_counter()
    E_occ, nit_occ, ok_occ, gamma, n, cj12, ck12 = occoptr(gamma, C, be, p)
    hist["t_occ"] += time.perf_counter() - t
    hist["E_occ"].append(E_occ)
    hist["nit_occ"].append(nit_occ)
    converged = False
    it = 0
    deadline = None if time_limit is None else t0 + time_limit
    for it in range(maxit):
        t = time.perf_counter()
        E_orb, C, nit_orb, ok_orb = orbopt_adam(gamma, C, be, p, state, deadline=deadline)
        t1 = time.perf_counter()
        E_occ, nit_occ, ok_occ, gamma, n, cj12, ck12 = occoptr(gamma, C, be, p)
        hist["t_orb"] += t1 - t
        hist["t_occ"] += time.perf_counter() - t1
        C, gamma = nof.order_occupations_softmax(C, gamma, p)
        g_orb = np.linalg.norm(calcorbg(np.zeros(p.nvar), n, cj12, ck12, C, be, p))
        if p.ndoc > 0 and getattr(be, "occupations", "host") != "host" and nof.native_occ_ok(p):
            g_occ = np.linalg.norm(be.occ_gradient(gamma, C))
        else:
            J_MO, K_MO, H_core = be.jkh_mo(C)
            if nof.native_occ_ok(p):
                g_occ = np.linalg.norm(nof.OccFunction(J_MO, K_MO, H_core, p)(gamma)[1])
            else:
                g_occ = np.linalg.norm(nof.calcoccg_fast(gamma, J_MO, K_MO, H_core, p))
        for k, v in (("E_orb", E_orb), ("E_occ", E_occ), ("g_orb", g_orb), ("g_occ", g_occ), ("nit_orb", nit_orb),
                     ("nit_occ", nit_occ), ("precision", be.precision)):
            hist[k].append(v)
        if callback is not None:
            callback(it, hist)
        while rungs and g_orb < rungs[0][0]:
            _, prec, ns = rungs.pop(0)
            be.set_precision(prec, ns)
        if (ok_orb or g_orb < tol) and (ok_occ or g_occ < tol):
            converged = True
            break
        if time_limit is not None and time.perf_counter() - t0 > time_limit:
            break
    n, _ = nof.ocupacion_softmax(gamma, p)
    cj12, ck12 = nof.cjckd8(n, p)
    if final_fp64 and be.precision != "fp64":
        be.set_precision("fp64")
    elag, Hmat = be.lagrange2(C, n, cj12, ck12)
    P = p.nbf5
    E = float(np.trace(elag[:P, :P]) + np.dot(n[:P], np.diagonal(Hmat)[:P]))
    return SolveResult(E, C, gamma, n, it + 1, converged, hist, time.perf_counter() - t0)
