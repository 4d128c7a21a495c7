"""Continuous-batching server for NOF solves on one GPU.

Requests (one synthetic molecule each: nbf, seed) arrive as a Poisson stream.
The admission loop admits the oldest waiting request that fits: a free slot
and an HBM reservation (b, its sliced copy and the peak workspace of the
device calls) within the budget.  Every admitted request runs the full NOF
solve (:func:`pynof_gb300.solver.solve`) in a worker thread with its own CUDA
stream, so requests that arrive while others are on the GPU join as slots and
memory free up and their kernels overlap on the device.  State (b, sliced b,
H, orbitals on the host) stays resident for the whole solve.  Latency is
arrival -> result; the report gives p50/p99 latency and solves/s.
"""
from __future__ import annotations

import dataclasses
import math
import threading
import time

import numpy as np
import torch

from . import _lib, nof, solver, synthetic


@dataclasses.dataclass
class Request:
    rid: int
    nbf: int
    seed: int
    arrival: float = 0.0  # seconds after the stream starts


@dataclasses.dataclass
class Result:
    rid: int
    nbf: int
    E_elec: float
    converged: bool
    iterations: int
    arrival: float
    admitted: float
    finished: float
    reserved_bytes: int

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def poisson_stream(count: int, rate: float, nbf_lo: int = 24, nbf_hi: int = 600, seed: int = 11):
    """count requests, nbf log-uniform in [nbf_lo, nbf_hi], exponential gaps."""
    rng = np.random.Generator(np.random.PCG64(seed))
    gaps = rng.exponential(1.0 / rate, count)
    t = np.cumsum(gaps) - gaps[0]
    sizes = np.exp(rng.uniform(math.log(nbf_lo), math.log(nbf_hi), count)).round().astype(int)
    return [Request(i, int(sizes[i]), 1000 + i, float(t[i])) for i in range(count)]


def reservation_bytes(st, precision: str, nslices: int) -> int:
    """HBM a solve holds: b, H, the sliced b and the largest workspace."""
    N, Q, P = st.nbf, st.nbfaux, st.nbf5
    b = N * N * Q * 8 + 2 * N * N * 8
    if precision == "mixed":
        prep = _lib.query("gb_ri_prepare_bytes_mixed", N, Q, nslices)
        ws = max(_lib.query("gb_jkh_mo_ri_workspace_mixed", N, P, Q, nslices),
                 _lib.query("gb_lagrange2_ri_workspace_mixed", N, P, Q, nslices))
    else:
        prep = 0
    # the FP64 path is also used after the precision switch
    ws64 = max(_lib.query("gb_jkh_mo_ri_workspace_f64", N, P, Q), _lib.query("gb_lagrange2_ri_workspace_f64", N, P, Q))
    ws = max(ws64, ws if precision == "mixed" else 0)
    out = 2 * N * N * 8 + N * P * 8 + 4 * P * P * 8
    return int(b + prep + ws + out)


class Server:
    """Continuous-batching NOF solve server.

    precision "mixed": the split-product path (``nslices`` digits; six are
    FP64-class, so by default no switch is made during the solve and only the
    closing Lagrangian, i.e. the reported energy, is evaluated on the FP64
    path, ``final_fp64``); ``fp64_switch`` or ``ladder`` (see
    :func:`pynof_gb300.solver.solve`) switch precision up as the orbital
    gradient falls.  precision "fp64": the plain DMMA path throughout.
    ``time_limit`` bounds each solve (seconds of its own wall time).

    ``occupations`` chooses where each solve's occupation CG runs.
    "device_sync" (the default here) runs the device kernels driven from the
    host in replays of eight evaluations, which share the GPU evenly with
    the other requests' GEMMs: on a config-5 stream (6 concurrent solves) it
    served 14.0 orbital steps/s with 3 requests converged, against 10.2 and 2
    for "host" (scipy's CG over the compiled evaluation on the host cores)
    and 6.3 and 1 for "device" (the conditional-node graph, the default of a
    single solve, whose device-side loop is served ahead of the other
    requests' work)."""

    def __init__(self, hbm_budget: float = 150e9, slots: int = 8, precision: str = "mixed", nslices: int = 6,
                 fp64_switch: float | None = None, tol: float = 1e-5, maxit: int = 200, device=None,
                 ladder=None, final_fp64: bool = True, time_limit: float | None = None,
                 occupations: str = "device_sync"):
        self.budget = int(hbm_budget)
        self.slots = slots
        self.precision = precision
        self.nslices = nslices
        self.fp64_switch = fp64_switch if precision == "mixed" else None
        self.ladder = ladder if precision == "mixed" else None
        self.final_fp64 = final_fp64 and precision == "mixed"
        self.time_limit = time_limit
        self.occupations = occupations
        self.tol = tol
        self.maxit = maxit
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self._lock = threading.Lock()
        self._cv = threading.Condition(self._lock)
        self.reserved = 0
        self.active = 0
        self.peak_reserved = 0
        self.peak_active = 0
        self.results: list[Result] = []
        self.errors: list[tuple[int, str]] = []
        self.steps = 0  # orbital steps (device Lagrangian evaluations) of finished solves
        # summed over finished solves: seconds in the occupation CG and in the
        # orbital-step loops, and the CG iterations
        self.t_occ = 0.0
        self.t_orb = 0.0
        self.cg_iterations = 0
        self.solve_fn = self.solve_request

    def _note_steps(self, k: int, t_occ: float = 0.0, t_orb: float = 0.0, cg_iterations: int = 0):
        with self._lock:
            self.steps += k
            self.t_occ += t_occ
            self.t_orb += t_orb
            self.cg_iterations += cg_iterations

    def solve_request(self, req: Request):
        """Full NOF solve of one request on its own stream: (E, converged, iterations)."""
        torch.cuda.set_device(self.device)
        st = synthetic.Structure.for_nbf(req.nbf)
        b, C, H, _ = synthetic.make_inputs(st, req.seed)
        be = solver.Backend(st, b, H, precision=self.precision, nslices=self.nslices, device=self.device,
                            occupations=self.occupations)
        res = solver.solve(be, C, nof.gamma_guess_softmax(st), st, tol=self.tol, maxit=self.maxit,
                           fp64_switch=self.fp64_switch, ladder=self.ladder, final_fp64=self.final_fp64,
                           time_limit=self.time_limit)
        be.stream.synchronize()
        self._note_steps(be.calls["lagrange2"], res.history["t_occ"], res.history["t_orb"],
                         int(np.sum(res.history["nit_occ"])))
        return res.E_elec, res.converged, res.iterations

    # ---- one solve -----------------------------------------------------
    def _solve(self, req: Request, t0: float, admitted: float, need: int):
        try:
            E, conv, iters = self.solve_fn(req)
            r = Result(req.rid, req.nbf, E, conv, iters, req.arrival, admitted, time.perf_counter() - t0, need)
            with self._lock:
                self.results.append(r)
        except Exception as e:  # a failing request fails alone; the others continue
            with self._lock:
                self.errors.append((req.rid, f"{type(e).__name__}: {e}"))
        finally:
            with self._cv:
                self.reserved -= need
                self.active -= 1
                self._cv.notify_all()

    # ---- the admission loop --------------------------------------------
    def run(self, requests: list[Request], realtime: bool = True) -> dict:
        pending: list[Request] = []
        arrivals = sorted(requests, key=lambda r: r.arrival)
        threads = []
        t0 = time.perf_counter()
        i = 0
        while i < len(arrivals) or pending:
            now = time.perf_counter() - t0
            while i < len(arrivals) and (not realtime or arrivals[i].arrival <= now):
                pending.append(arrivals[i])
                i += 1
            admitted_any = False
            with self._cv:
                for req in list(pending):
                    need = reservation_bytes(synthetic.Structure.for_nbf(req.nbf), self.precision, self.nslices)
                    if need > self.budget:
                        pending.remove(req)
                        self.errors.append((req.rid, f"needs {need} bytes, above the {self.budget}-byte budget"))
                        continue
                    if self.active < self.slots and self.reserved + need <= self.budget:
                        pending.remove(req)
                        self.reserved += need
                        self.active += 1
                        self.peak_reserved = max(self.peak_reserved, self.reserved)
                        self.peak_active = max(self.peak_active, self.active)
                        th = threading.Thread(target=self._solve, args=(req, t0, time.perf_counter() - t0, need),
                                              daemon=True)
                        th.start()
                        threads.append(th)
                        admitted_any = True
                if not admitted_any:
                    wait = 0.05
                    if i < len(arrivals) and realtime:
                        wait = max(0.0, min(wait, arrivals[i].arrival - (time.perf_counter() - t0)))
                    self._cv.wait(timeout=wait)
        for th in threads:
            th.join()
        wall = time.perf_counter() - t0
        lat = np.array([r.latency for r in self.results]) if self.results else np.array([float("nan")])
        conv = [r for r in self.results if r.converged]
        clat = np.array([r.latency for r in conv]) if conv else np.array([float("nan")])
        return {
            "requests": len(requests), "completed": len(self.results), "failed": len(self.errors),
            "wall_s": wall, "solves_per_s": len(self.results) / wall,
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "converged": len(conv), "converged_per_s": len(conv) / wall,
            "p50_latency_converged_s": float(np.percentile(clat, 50)),
            "p99_latency_converged_s": float(np.percentile(clat, 99)),
            "orbital_steps_per_s": self.steps / wall,
            "occupation_cg_s": self.t_occ, "orbital_loops_s": self.t_orb, "occupation_cg_iterations": self.cg_iterations,
            "occupations": self.occupations,
            "peak_active": self.peak_active, "peak_reserved_gb": self.peak_reserved / 1e9,
            "precision": self.precision, "slots": self.slots, "budget_gb": self.budget / 1e9,
            "time_limit_s": self.time_limit,
        }
