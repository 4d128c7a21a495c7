#!/usr/bin/env python
"""JK-build throughput benchmark (one JSON line on rank 0).

Workload: one RI JK build = computeJKj (J_i, K_i for all i < nbf5) at
nbf=600, naux=2400, nbf5=300 (seeded synthetic inputs; b is 6.9 GB, larger
than L2, so no flush is needed between steps).

Legs of the default run (``--impl ours``):
  value   builds/s with b, C resident in HBM (device-timed, CUDA events), on
          the split-product tensor-core path (6 bf16 digit slices, FP64-class
          accuracy; ``--precision fp64`` times the DMMA path instead);
  fp64    the plain FP64 DMMA path on the same inputs (builds/s) and the
          errors of the headline path against it: J, K normwise and the
          electronic energy assembled from J, K (the no1 > 0 route of
          ENERGY1r, closed shell) in FP64;
  e2e     builds/s through the reference-facing drop-in call
          ``pynof_gb300.integrals.JKj_RI_GPU(C, b, p)``: host C in (pinned),
          host J, K out (pinned), copies inside the timed region;
  roofline  the dominant kernel's algorithmic rate over the launch time the
          library's event profiler recorded inside the timed region;
  cpu_baseline  the CPU oracle (numpy/OpenBLAS, all host threads): whole
          builds at the same configuration (median of --cpu-reps).

``--impl reference`` times the CPU restatement of PyNOF's JKj_RI (the
reference itself is Python and is not present at run time) on the same
workload; rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOAD = "c3"
METRIC = "RI-JK builds/s at nbf=600 (computeJKj, J_i and K_i for i < nbf5)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--cpu-reps", type=int, default=3, help="whole CPU-oracle builds timed for cpu_baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--nslices", type=int, default=6)
    ap.add_argument("--fp64-steps", type=int, default=2, help="steps of the FP64 comparison leg (0 = skip)")
    ap.add_argument("--mode", choices=["jk", "batch", "serve", "precision", "mo", "hostlink", "occ"], default="jk",
                    help="jk: one nbf=600 build (the headline); batch: 64 molecules; serve: NOF solve stream; "
                         "precision: every split form against FP64 (J, K, E, orbital gradient); "
                         "mo: computeJKH_MO and computeLagrange2 per kernel, with the bandwidth kernels' GB/s; "
                         "hostlink: device <-> pinned host copy rates at the size of one build's J, K; "
                         "occ: occoptr's CG on the device against scipy's on the host")
    ap.add_argument("--nmol", type=int, default=64)
    ap.add_argument("--batch-nbf-max", type=int, default=400, help="largest nbf of the batch (batch mode)")
    ap.add_argument("--requests", type=int, default=16)
    ap.add_argument("--rate", type=float, default=10.0)
    ap.add_argument("--nbf-min", type=int, default=24)
    ap.add_argument("--nbf-max", type=int, default=150)
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--tol", type=float, default=1e-5)
    ap.add_argument("--maxit", type=int, default=200)
    ap.add_argument("--time-limit", type=float, default=None, help="seconds per served solve (serve mode)")
    ap.add_argument("--occ-nbf", default="60,300,600", help="nbf of the occupation problems (occ mode)")
    ap.add_argument("--occupations", choices=["host", "device", "device_sync"], default="device_sync",
                    help="where served solves run the occupation CG (serve mode)")
    ap.add_argument("--serve-paths", default="mixed,fp64", help="precisions served in turn (serve mode)")
    return ap.parse_args()


def flops_jkj(N, P, Q):
    """Algorithmic flops of one RI JK build in the reference's formulation:
    2PN^2Q (half transform) + 2PNQ (diagonal) + 2PN^2Q (J) + 2PN^2Q (K)."""
    return 6.0 * P * N * N * Q + 2.0 * P * N * Q


KERNEL_FLOPS = {
    # FP64 flops per launch in the reference formulation (symmetry the kernels
    # exploit is not discounted)
    "gemm_f64:half_transform": lambda N, P, Q: 2.0 * P * N * N * Q,
    "gemm_f64:J": lambda N, P, Q: 2.0 * P * N * N * Q,
    "gemm_f64:K": lambda N, P, Q: 2.0 * P * N * N * Q,
    "contract_diag": lambda N, P, Q: 2.0 * P * N * Q,
    "ozaki_tc:half_transform": lambda N, P, Q: 2.0 * P * N * N * Q,
    "ozaki_tc:J": lambda N, P, Q: 2.0 * P * N * N * Q,
    "ozaki_tc:K": lambda N, P, Q: 2.0 * P * N * N * Q,
}


def n_products(S):
    """bf16 slice products per FP64 product: pairs (s, t) with s + t <= S + 1."""
    return S * (S + 1) // 2


def energy_from_jk(J, K, C, H, n, cj, ck):
    """Closed-shell electronic energy from J_i, K_i (FP64, numpy):
    E = sum_i C_i^T F_i C_i + sum_i n_i H_ii with the generalized Fock
    F_i = n_i H + n_i J_i + sum_j cj_ij J_j - sum_j ck_ij K_j (zero diagonals),
    i.e. computeF_RC -> computeLagrange -> computeE_elec with no1 = 0."""
    P = J.shape[0]
    Cp = C[:, :P]
    Hd = np.einsum("mi,mi->i", Cp, H @ Cp)
    Jd = np.einsum("mi,jmi->ji", Cp, np.matmul(J, Cp))
    Kd = np.einsum("mi,jmi->ji", Cp, np.matmul(K, Cp))
    cj = cj.copy()
    ck = ck.copy()
    np.fill_diagonal(cj, 0.0)
    np.fill_diagonal(ck, 0.0)
    return float(2.0 * np.dot(n, Hd) + np.dot(n, np.diagonal(Jd)) + np.sum(cj * Jd.T) - np.sum(ck * Kd.T))


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]

    def __init__(self, gpu_id: str):
        self.gpu_id = gpu_id
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", self.gpu_id, "--query-gpu=" + ",".join(self.FIELDS), "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cpu_baseline(b, C, P, N, Q, reps=3):
    """The oracle's JKj_RI (numpy/OpenBLAS, every host thread) over all nbf5
    orbitals: builds/s (median of ``reps`` whole builds) and the last build's
    J, K, which the accuracy legs compare against."""
    from oracle import pynof_oracle as orc

    cores = os.cpu_count()
    orc.jkj_ri(C, b, 2)  # warm the BLAS threads
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        J, K = orc.jkj_ri(C, b, P)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    rec = {"value": 1.0 / t, "unit": "builds/s", "cores": cores, "kind": "port",
           "sample": f"whole builds (J_i, K_i for all {P} orbitals) at nbf={N}, naux={Q}, median of {reps}; "
                     "numpy/OpenBLAS restatement of JKj_RI",
           "seconds_per_build": t}
    return rec, J, K


def make_workload(name):
    from pynof_gb300 import synthetic

    st = synthetic.structure(name)
    b, C, H, n = synthetic.make_inputs(st, 0)
    return st, b, C, H, n


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    st, b, C, H, n = make_workload(args.workload)
    N, P, Q = st.nbf, st.nbf5, st.nbfaux
    from oracle import pynof_oracle as orc

    orc.jkj_ri(C, b, 2)
    for _ in range(args.warmup):
        orc.jkj_ri(C, b, P)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.jkj_ri(C, b, P)
    dt = time.perf_counter() - t0
    value = args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "builds/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"RI JK build nbf={N} naux={Q} nbf5={P} (computeJKj)"},
        "cpu_baseline": {"value": value, "unit": "builds/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": f"one whole build (J_i, K_i for all {P} orbitals) per step; numpy/OpenBLAS "
                                   "restatement of JKj_RI on every host thread"},
        "e2e": {"value": value, "unit": "builds/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    from pynof_gb300 import _lib, integrals, ops
    from pynof_gb300.replicas import Replicas

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    reps = Replicas(device=dev)
    world, rank = reps.world, reps.rank

    st, b, C, H, n = make_workload(args.workload)
    N, P, Q = st.nbf, st.nbf5, st.nbfaux
    db = ops.to_device(b)
    dC = ops.to_device(C)
    ops.check_device_status()
    asym = ops.check_symmetric(db)
    assert asym == 0.0, asym
    barrier = reps.barrier

    mixed = args.precision == "mixed"
    S = args.nslices
    integrals.set_precision(args.precision, S)

    def build():
        if mixed:
            return ops.jkj_ri_mixed(dC, prep, P)
        return ops.jkj_ri(dC, db, P)

    # ---- one-time preparation of the resident sliced factor --------------
    prep = None
    prep_s = 0.0
    if mixed:
        barrier()
        t0 = time.perf_counter()
        prep = integrals.prepared(db, S)
        barrier()
        prep_s = time.perf_counter() - t0

    # ---- device-resident leg --------------------------------------------
    for _ in range(args.warmup):
        J, K = build()
    if mixed:
        ops.check_device_status()
    del J, K
    props = torch.cuda.get_device_properties(dev)
    gpu_id = str(getattr(props, "uuid", local))
    if gpu_id and not gpu_id.startswith("GPU-") and len(gpu_id) == 36:
        gpu_id = "GPU-" + gpu_id
    clocks = ClockSampler(gpu_id)
    barrier()
    clocks.start()
    _lib.profile_start()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        J, K = build()
    e1.record(stream)
    barrier()
    prof = _lib.profile_stop()
    clk = clocks.stop()
    if mixed:
        ops.check_device_status()
    value, dev_s = reps.throughput(args.steps, e0.elapsed_time(e1) / 1e3)

    # ---- end-to-end leg through the drop-in call -------------------------
    C_pin = torch.from_numpy(C).pin_memory().numpy()
    p = st
    for _ in range(max(1, args.warmup)):
        Jh, Kh = integrals.JKj_RI_GPU(C_pin, db, p)
    del Jh, Kh
    barrier()
    t0 = time.perf_counter()
    step_s = []
    for _ in range(args.steps):
        ts = time.perf_counter()
        Jh, Kh = integrals.JKj_RI_GPU(C_pin, db, p)
        step_s.append(time.perf_counter() - ts)
    barrier()
    e2e_value, e2e_s = reps.throughput(args.steps, time.perf_counter() - t0)
    h2d = C.nbytes
    d2h = 2 * P * N * N * 8
    del Jh, Kh

    # ---- computeJKH_MO and computeLagrange2 (what the solve loop calls) ---
    from pynof_gb300 import nof

    dH = ops.to_device(H)
    dn = ops.to_device(n)
    cj_h, ck_h = nof.cjckd8(n, st)
    np.fill_diagonal(cj_h, 0.0)
    np.fill_diagonal(ck_h, 0.0)
    dcj, dck = ops.to_device(cj_h), ops.to_device(ck_h)

    def timed(fn, count):
        fn()
        barrier()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(count):
            fn()
        t1.record(stream)
        barrier()
        return count * world / reps.max(t0.elapsed_time(t1) / 1e3)

    rates = {"unit": "calls/s", "jkh_mo_per_s": {}, "lagrange2_per_s": {}}
    if mixed:
        rates["jkh_mo_per_s"]["mixed"] = timed(lambda: ops.jkh_mo_ri_mixed(dC, dH, prep, P), args.steps)
        rates["lagrange2_per_s"]["mixed"] = timed(
            lambda: ops.lagrange2_ri_mixed(dC, dH, prep, dn, dcj, dck, P, st.nbeta, st.nalpha), args.steps)
        ops.check_device_status()
    if args.fp64_steps > 0 or not mixed:
        k64 = max(1, args.fp64_steps)
        rates["jkh_mo_per_s"]["fp64"] = timed(lambda: ops.jkh_mo_ri(dC, dH, db, P), k64)
        rates["lagrange2_per_s"]["fp64"] = timed(
            lambda: ops.lagrange2_ri(dC, dH, db, dn, dcj, dck, P, st.nbeta, st.nalpha), k64)

    # ---- FP64 DMMA comparison leg -----------------------------------------
    fp64 = None
    J64h = K64h = None
    if mixed and args.fp64_steps > 0:
        J64, K64 = ops.jkj_ri(dC, db, P)
        barrier()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.fp64_steps):
            J64, K64 = ops.jkj_ri(dC, db, P)
        f1.record(stream)
        barrier()
        fp64_s = reps.max(f0.elapsed_time(f1) / 1e3)
        fp64 = {"value": world * args.fp64_steps / fp64_s, "unit": "builds/s", "steps": args.fp64_steps,
                "ms_per_step": 1e3 * fp64_s / args.fp64_steps,
                "speedup_of_headline": value / (world * args.fp64_steps / fp64_s)}
        J64h, K64h = J64.cpu().numpy(), K64.cpu().numpy()
        del J64, K64
    Jh, Kh = J.cpu().numpy(), K.cpu().numpy()
    del J, K
    torch.cuda.empty_cache()

    # ---- CPU oracle: baseline rate and the accuracy of both device paths ---
    cpu = accuracy = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import pynof_oracle as orc

        cpu, Jr, Kr = cpu_baseline(b, C, P, N, Q, reps=args.cpu_reps)
        t0 = time.perf_counter()
        orc.jkh_mo_ri(C, H, b, P)
        cpu["jkh_mo_per_s"] = 1.0 / (time.perf_counter() - t0)
        t0 = time.perf_counter()
        orc.lagrange2(n, cj_h.copy(), ck_h.copy(), C, H, None, b, st)
        cpu["lagrange2_per_s"] = 1.0 / (time.perf_counter() - t0)
        rates["jkh_mo_per_s"]["cpu_oracle"] = cpu["jkh_mo_per_s"]
        rates["lagrange2_per_s"]["cpu_oracle"] = cpu["lagrange2_per_s"]

        def nrel(a, r):
            return float(np.max(np.abs(a - r)) / np.max(np.abs(r)))

        E_ref = energy_from_jk(Jr, Kr, C, H, n, cj_h, ck_h)
        accuracy = {"reference": "the CPU oracle (numpy FP64 restatement of JKj_RI) on the same inputs",
                    "energy_definition": "closed-shell E from J_i, K_i: computeF_RC -> computeLagrange -> "
                                         "computeE_elec with GNOF cj12, ck12 (zero diagonals), no1 = 0",
                    "E_oracle_hartree": E_ref, "headline": {
                        "J_normwise_err": nrel(Jh, Jr), "K_normwise_err": nrel(Kh, Kr),
                        "E_abs_err_hartree": abs(energy_from_jk(Jh, Kh, C, H, n, cj_h, ck_h) - E_ref)}}
        if J64h is not None:
            accuracy["fp64_dmma"] = {"J_normwise_err": nrel(J64h, Jr), "K_normwise_err": nrel(K64h, Kr),
                                     "E_abs_err_hartree": abs(energy_from_jk(J64h, K64h, C, H, n, cj_h, ck_h) -
                                                              E_ref)}
        del Jr, Kr
    if fp64 is not None and accuracy is not None:
        fp64["E_abs_err_hartree_vs_oracle"] = accuracy["fp64_dmma"]["E_abs_err_hartree"]

    # ---- roofline of the dominant kernel ---------------------------------
    peaks, peak_src = measured_peaks()
    top = max(prof.items(), key=lambda kv: kv[1][1])
    name, (launches, total_ms) = top
    per_launch_s = total_ms / 1e3 / launches
    fl = KERNEL_FLOPS.get(name, lambda N, P, Q: float("nan"))(N, P, Q)
    traffic = None
    if name == "ozaki_tc:half_transform" and S <= 6:
        # DRAM bytes per launch: an ncu capture of this kernel at nbf=300 read
        # 1.316 GB + wrote 0.409 GB for 1.745 GB of algorithmic bytes (b's
        # digit planes once + T written; part of T's writes still sit in L2 at
        # the end of the launch); the same ratio applied to this workload's bytes
        kpad = -(-N // 16) * 16
        alg_bytes = float(N) * Q * kpad * 2 * S + 8.0 * P * N * Q
        traffic = 0.9883 * alg_bytes
    if name.startswith("ozaki_tc"):
        tensor_fl = n_products(S) * fl
        achieved = tensor_fl / per_launch_s / 1e12
        peak = float(peaks["bf16_tflops"])
        roof = {"bound": "tensor", "kernel": name, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": traffic,
                "traffic_note": None if traffic is None else (
                    "bytes per launch, scaled from dram__bytes_read.sum + dram__bytes_write.sum of the same kernel "
                    f"at nbf=300 (ncu) by the algorithmic bytes ({alg_bytes:.4g} here)"),
                "peak_source": f"bf16_tflops of {peak_src} MEASURED_PEAKS.json (burst; kernel timed alone)",
                "achieved_definition": f"{n_products(S)} bf16 slice products x reference-formulation flops "
                                       "of the launch / launch time",
                "fp64_equivalent_tflops": fl / per_launch_s / 1e12}
    else:
        fp64_peak = measure_dgemm_tflops(torch, dev)
        achieved = fl / per_launch_s / 1e12
        roof = {"bound": "tensor", "kernel": name, "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": achieved / fp64_peak, "traffic": None,
                "peak_source": "cuBLAS DGEMM 8192^3 measured in this run (FP64 pipe; no FP64 figure is "
                               "in MEASURED_PEAKS.json)"}
    roof.update({"flops_per_launch_fp64": fl, "ms_per_launch": 1e3 * per_launch_s,
                 "kernels": {k: {"launches": v[0], "total_ms": round(v[1], 3)} for k, v in prof.items()}})

    line = {
        "metric": METRIC, "value": value, "unit": "builds/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16-split-f64" if mixed else "f64", "data": "synthetic",
        "config": {"workload": f"RI JK build nbf={N} naux={Q} nbf5={P} (computeJKj)",
                   "precision": f"mixed nslices={S} ({n_products(S)} bf16 products)" if mixed else "fp64",
                   "l2": "inputs larger than L2 (b = %.1f GB)" % (b.nbytes / 1e9),
                   "parallelism": f"replicas x{world}",
                   "prepare_s": round(prep_s, 4)},
        "e2e": {"value": e2e_value, "unit": "builds/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": {"median": 1e3 * statistics.median(step_s), "min": 1e3 * min(step_s),
                                "max": 1e3 * max(step_s)}},
        "roofline": roof,
        "gpu_launches": sum(v[0] for v in prof.values()),
        "clocks": clk,
        "fp64_path": fp64,
        "hot_path_rates": rates,
        "accuracy": accuracy,
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line), flush=True)
    reps.close()


def measure_dgemm_tflops(torch, dev, n=8192, reps=3):
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    bm = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, bm)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, bm)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return 2.0 * n ** 3 / best / 1e12


def run_batch(args):
    """64 molecules, nbf log-uniform in [24, 400], naux = 4 nbf, nbf5 ~ nbf/2:
    one batched build (grouped launches in a CUDA graph, autotuned tiles)
    against 64 sequential single-molecule builds (FP64 and mixed)."""
    import torch

    from pynof_gb300 import batch as bmod
    from pynof_gb300 import ops, synthetic

    torch.cuda.set_device(0)
    sizes = synthetic.batch_sizes(args.nmol, hi=args.batch_nbf_max)
    mols, fp64_in = [], []
    for i, nbf in enumerate(sizes):
        st = synthetic.Structure.for_nbf(nbf)
        b, C, H, n = synthetic.make_inputs(st, 1000 + i)
        db, dC = ops.to_device(b), ops.to_device(C)
        mols.append((dC, ops.PreparedRI(db, args.nslices), st.nbf5))
        fp64_in.append((dC, db, st.nbf5))
    torch.cuda.synchronize()
    flops = sum(flops_jkj(m[1].nbf, m[2], m[1].naux) for m in mols)

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps

    t64 = timed(lambda: [ops.jkj_ri(c, bb, p) for c, bb, p in fp64_in], 1)
    tmx = timed(lambda: [ops.jkj_ri_mixed(c, pr, p) for c, pr, p in mols], args.steps)
    tiles, info = bmod.autotune(mols, reps=2, use_cache=False)
    plan = bmod.BatchJK(mols, tiles=tiles)
    stream = plan.stream
    plan.run()
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        plan.run()
    e1.record(stream)
    e1.synchronize()
    tgr = e0.elapsed_time(e1) / 1e3 / args.steps
    ops.check_device_status()
    # accuracy of the batched build against the FP64 builds
    err = 0.0
    for (c, bb, p), J, K in zip(fp64_in, plan.J, plan.K):
        J64, K64 = ops.jkj_ri(c, bb, p)
        err = max(err, float((J - J64).abs().max() / J64.abs().max()), float((K - K64).abs().max() / K64.abs().max()))
    nm = len(mols)
    line = {"metric": f"batched RI-JK builds/s, {args.nmol} molecules nbf log-uniform in [24,{args.batch_nbf_max}]",
            "unit": "builds/s",
            "value": nm / tgr, "steps": args.steps, "dtype": "bf16-split-f64", "data": "synthetic",
            "config": {"workload": f"{nm} molecules, nbf {min(sizes)}..{max(sizes)} (median "
                                   f"{int(np.median(sizes))}), naux=4 nbf, nbf5=5 (nbf//10)",
                       "nslices": args.nslices, "tiles": list(tiles), "autotune": info.get("timings")},
            "grouped_graph_s": tgr, "sequential_mixed_s": tmx, "sequential_fp64_s": t64,
            "speedup_vs_sequential_mixed": tmx / tgr, "speedup_vs_sequential_fp64": t64 / tgr,
            "fp64_equivalent_tflops": flops / tgr / 1e12, "max_normwise_err_vs_fp64": err}
    print(json.dumps(line), flush=True)


def run_serve(args):
    """A Poisson stream of full NOF solves, continuous batching: the mixed
    path (six digit slices, closing Lagrangian on the FP64 path) against the
    plain FP64 path, on the same requests."""
    import torch

    from pynof_gb300 import serve

    torch.cuda.set_device(0)
    reqs = serve.poisson_stream(args.requests, args.rate, args.nbf_min, args.nbf_max, seed=11)
    out = {}
    paths = args.serve_paths.split(",")
    for prec in paths:
        srv = serve.Server(hbm_budget=150e9, slots=args.slots, precision=prec, nslices=args.nslices,
                           tol=args.tol, maxit=args.maxit, final_fp64=True, time_limit=args.time_limit,
                           occupations=args.occupations)
        out[prec] = srv.run(reqs)
        out[prec]["energies"] = {r.rid: r.E_elec for r in srv.results if r.converged}
    both = [k for k in out.get("fp64", {}).get("energies", {}) if k in out.get("mixed", {}).get("energies", {})]
    dE = max((abs(out["mixed"]["energies"][k] - out["fp64"]["energies"][k]) for k in both), default=float("nan"))
    for prec in out:
        out[prec].pop("energies")
    line = {"metric": "served NOF solves: p50/p99 latency and solves/s", "unit": "solves/s",
            "value": out[paths[0]]["solves_per_s"], "data": "synthetic",
            "config": {"requests": args.requests, "rate_per_s": args.rate,
                       "nbf": f"log-uniform {args.nbf_min}..{args.nbf_max}",
                       "naux": "4 nbf", "tol": args.tol, "maxit": args.maxit, "slots": args.slots,
                       "hbm_budget_gb": 150, "time_limit_per_solve_s": args.time_limit,
                       "occupation_cg": args.occupations,
                       "precision_switch": "six digit slices (FP64-class) throughout; closing Lagrangian "
                                           "(reported energy) on the FP64 path"},
            "mixed": out.get("mixed"), "plain_fp64": out.get("fp64"),
            "max_abs_dE_mixed_vs_fp64_hartree": dE, "dE_over_requests_converged_in_both": len(both)}
    print(json.dumps(line), flush=True)


def run_precision(args):
    """Each arithmetic form of the path on the same seeded inputs: JK builds/s
    (computeJKj) and computeLagrange2 calls/s, with the errors of J, K, the
    energy E = tr elag[:P,:P] + sum_i n_i Hmat_ii and the packed orbital
    gradient 4 (elag - elag^T) against the FP64 (DMMA) path."""
    import torch

    from pynof_gb300 import nof, ops

    torch.cuda.set_device(0)
    st, b, C, H, n = make_workload(args.workload)
    N, P, Q = st.nbf, st.nbf5, st.nbfaux
    db, dC, dH, dn = (ops.to_device(x) for x in (b, C, H, n))
    cj, ck = nof.cjckd8(n, st)
    np.fill_diagonal(cj, 0.0)
    np.fill_diagonal(ck, 0.0)
    dcj, dck = ops.to_device(cj), ops.to_device(ck)
    iu, ju = np.triu_indices(N, 1)
    keep = iu < P

    def timed(fn, reps):
        out = fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            out = fn()
        e1.record()
        torch.cuda.synchronize()
        return out, e0.elapsed_time(e1) / 1e3 / reps

    def energy_grad(elag, Hmat):
        el = elag.cpu().numpy()
        E = float(np.trace(el[:P, :P]) + np.dot(n[:P], np.diagonal(Hmat.cpu().numpy())[:P]))
        g = 4.0 * (el - el.T)
        return E, g[iu[keep], ju[keep]]

    def nrel(a, r):
        return float((a - r).abs().max() / r.abs().max())

    forms = [("fp64", None), ("mixed_s6", 6), ("bf16x3", 2), ("tf32x3", ops.SPLIT_TF32X3)]
    out, ref = {}, None
    for name, code in forms:
        if code is None:
            (J, K), t_jk = timed(lambda: ops.jkj_ri(dC, db, P), 1)
            (JM, KM, Hc), t_mo = timed(lambda: ops.jkh_mo_ri(dC, dH, db, P), 1)
            (el, Hm), t_l2 = timed(lambda: ops.lagrange2_ri(dC, dH, db, dn, dcj, dck, P, st.nbeta, st.nalpha), 1)
        else:
            prep = ops.PreparedRI(db, code)
            (J, K), t_jk = timed(lambda: ops.jkj_ri_mixed(dC, prep, P), args.steps)
            (JM, KM, Hc), t_mo = timed(lambda: ops.jkh_mo_ri_mixed(dC, dH, prep, P), args.steps)
            (el, Hm), t_l2 = timed(lambda: ops.lagrange2_ri_mixed(dC, dH, prep, dn, dcj, dck, P, st.nbeta,
                                                                 st.nalpha), args.steps)
            ops.check_device_status()
            del prep
        E, g = energy_grad(el, Hm)
        rec = {"jk_builds_per_s": 1.0 / t_jk, "jkh_mo_per_s": 1.0 / t_mo, "lagrange2_per_s": 1.0 / t_l2,
               "E_hartree": E}
        if ref is None:
            ref = (J, K, JM, KM, E, g)
        else:
            J64, K64, JM64, KM64, E64, g64 = ref
            rec.update({
                "J_normwise_err": nrel(J, J64), "K_normwise_err": nrel(K, K64),
                "J_MO_normwise_err": nrel(JM, JM64), "K_MO_normwise_err": nrel(KM, KM64),
                "E_abs_err_hartree": abs(E - E64),
                "grad_normwise_err": float(np.abs(g - g64).max() / np.abs(g64).max()),
                "grad_max_abs_err": float(np.abs(g - g64).max()),
            })
        out[name] = rec
        del J, K, JM, KM, Hc, el, Hm
        torch.cuda.empty_cache()
    # the reference algorithm on the host cores (numpy / OpenBLAS restatement)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import pynof_oracle as orc

        orc.jkj_ri(C, b, 2)
        t0 = time.perf_counter()
        orc.jkj_ri(C, b, P)
        t_a1 = time.perf_counter() - t0
        t0 = time.perf_counter()
        orc.jkh_mo_ri(C, H, b, P)
        t_a3 = time.perf_counter() - t0
        t0 = time.perf_counter()
        orc.lagrange2(n, cj.copy(), ck.copy(), C, H, None, b, st)
        t_a5 = time.perf_counter() - t0
        cpu = {"cores": os.cpu_count(), "kind": "port",
               "sample": "computeJKj, computeJKH_MO and computeLagrange2, one whole call each",
               "jk_builds_per_s": 1.0 / t_a1, "jkh_mo_per_s": 1.0 / t_a3, "lagrange2_per_s": 1.0 / t_a5}
    line = {"metric": "precision forms of the RI JK build and Lagrangian vs FP64", "unit": "builds/s",
            "value": out["mixed_s6"]["jk_builds_per_s"], "data": "synthetic",
            "config": {"workload": f"nbf={N} naux={Q} nbf5={P}", "steps": args.steps,
                       "coefficients": "GNOF (PNOF8) cj12, ck12 from the synthetic occupations",
                       "reference": "FP64 DMMA path (parity-tested against the oracle at 1e-10)"},
            "forms": out, "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


def mo_kernel_bytes(N, P, Q, S):
    """Algorithmic DRAM bytes per call of each bandwidth-bound kernel of
    computeJKH_MO ("jkh") and computeLagrange2 ("lag2"): every input read once
    and every output written once (float64 = 8 B; a digit slicing reads 8 B and
    writes 2S B per element, its exponent pass reads the 8 B once more)."""
    dig = 8 + 2 * S
    jkh = {
        "slice_digits": (P * N + P * N * Q) * dig,
        "slice_rowexp": (P * N + P * N * Q) * 8,
        "gather_diag": 16 * P * Q,
        "row_sumsq": 8 * P * P * Q + 8 * P * P,
        "col_dot": 16 * N * P + 8 * P,
    }
    lag2 = {
        "slice_digits": (N * N + P * N * Q + N * P * Q + P * P * Q) * dig,
        "slice_rowexp": (N * N + P * N * Q + N * P * Q + P * P * Q) * 8,
        "gather_diag": 16 * P * Q,
        "copy_zero_diag": 16 * P * P,
        "add_scaled_rows": 24 * P * Q,
        "make_exchange_operand": 16 * P * P * Q + 8 * P * P,
        "lagrange2_hterm": 16 * N * N + 8 * N * P,
    }
    fused = dict(lag2)
    fused["row_sumsq"] = 8 * P * P * Q + 8 * P * P
    fused["col_dot"] = 16 * N * P + 8 * P
    return {"jkh": jkh, "lag2": lag2, "fused": fused}


def run_mo(args):
    """computeJKH_MO, computeLagrange2 and the two in one call (what each
    orbital step of the solver makes) on the split-product path at one
    workload: calls/s and, per kernel, ms per call; for the bandwidth-bound
    kernels their algorithmic bytes and GB/s against the measured HBM copy
    rate.  Times come from the library's event profiler (CUDA events on the
    launch stream) over --steps calls after --warmup."""
    import torch

    from pynof_gb300 import _lib, integrals, nof, ops

    torch.cuda.set_device(0)
    st, b, C, H, n = make_workload(args.workload)
    N, P, Q, S = st.nbf, st.nbf5, st.nbfaux, args.nslices
    db, dC, dH, dn = ops.to_device(b), ops.to_device(C), ops.to_device(H), ops.to_device(n)
    integrals.set_precision("mixed", S)
    prep = integrals.prepared(db, S)
    cj, ck = nof.cjckd8(n, st)
    np.fill_diagonal(cj, 0.0)
    np.fill_diagonal(ck, 0.0)
    dcj, dck = ops.to_device(cj), ops.to_device(ck)
    calls = {
        "jkh": lambda: ops.jkh_mo_ri_mixed(dC, dH, prep, P),
        "lag2": lambda: ops.lagrange2_ri_mixed(dC, dH, prep, dn, dcj, dck, P, st.nbeta, st.nalpha),
        "fused": lambda: ops.jkh_lagrange2_ri_mixed(dC, dH, prep, dn, dcj, dck, P, st.nbeta, st.nalpha),
    }
    peaks, peak_src = measured_peaks()
    hbm = peaks.get("hbm_gbs", 6800.0)
    nbytes = mo_kernel_bytes(N, P, Q, S)
    out = {}
    stream = torch.cuda.current_stream()
    for name, fn in calls.items():
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        _lib.profile_start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        prof = _lib.profile_stop()
        ops.check_device_status()
        ms = e0.elapsed_time(e1) / args.steps
        kern = {}
        for k, (launches, total) in sorted(prof.items(), key=lambda kv: -kv[1][1]):
            rec = {"launches_per_call": launches / args.steps, "ms_per_call": total / args.steps,
                   "share": total / args.steps / ms}
            if k in nbytes[name]:
                gbs = nbytes[name][k] / (total / args.steps * 1e-3) / 1e9
                rec.update({"bytes_per_call": nbytes[name][k], "gbs": gbs, "frac_of_hbm": gbs / hbm})
            kern[k] = rec
        out[name] = {"calls_per_s": 1e3 / ms, "ms_per_call": ms, "kernels": kern}
    line = {"mode": "mo", "metric": "computeJKH_MO and computeLagrange2 calls/s (split products, nslices=%d)" % S,
            "unit": "calls/s", "data": "synthetic",
            "config": {"workload": f"nbf={N} naux={Q} nbf5={P}", "steps": args.steps, "warmup": args.warmup},
            "hbm_peak_gbs": hbm, "peak_source": f"hbm_gbs of {peak_src} MEASURED_PEAKS.json",
            "computeJKH_MO": out["jkh"], "computeLagrange2": out["lag2"],
            "computeJKH_MO+computeLagrange2 (one call)": out["fused"]}
    print(json.dumps(line), flush=True)


def run_hostlink(args):
    """Copy rates between HBM and pinned host memory at the size of one
    nbf=600 build's J and K (2 x 864 MB), the transfer the e2e leg makes: one
    copy stream, two copy streams (one per array), and a device -> host copy
    after a device kernel has written the buffer (as in the build).  CUDA
    events on the copy streams, best of --steps.  Also the host's NUMA nodes
    and this process's CPU set."""
    import torch

    torch.cuda.set_device(0)
    n = 300 * 600 * 600
    dev = [torch.empty(n, dtype=torch.float64, device="cuda").fill_(1.0) for _ in range(2)]
    host = [torch.empty(n, dtype=torch.float64, pin_memory=True) for _ in range(2)]
    streams = [torch.cuda.Stream() for _ in range(2)]
    nbytes = 2 * n * 8

    def timed(two_streams: bool, d2h: bool):
        best = float("inf")
        for _ in range(max(1, args.steps)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for i in range(2):
                st = streams[i if two_streams else 0]
                with torch.cuda.stream(st):
                    (host[i].copy_(dev[i], non_blocking=True) if d2h else dev[i].copy_(host[i], non_blocking=True))
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        return nbytes / best / 1e9

    for _ in range(2):
        timed(False, True)
    out = {"d2h_gbs_one_stream": timed(False, True), "d2h_gbs_two_streams": timed(True, True),
           "h2d_gbs_one_stream": timed(False, False), "h2d_gbs_two_streams": timed(True, False)}
    nodes = sorted(d for d in os.listdir("/sys/devices/system/node") if d.startswith("node")) \
        if os.path.isdir("/sys/devices/system/node") else []
    line = {"mode": "hostlink", "bytes_per_copy": nbytes, "unit": "GB/s", "steps": args.steps,
            "numa_nodes": nodes, "cpus_of_process": len(os.sched_getaffinity(0)),
            "pinned": "torch pin_memory (cudaHostAlloc)", **out}
    print(json.dumps(line), flush=True)


def run_occ(args):
    """occoptr's minimisation over gamma (scipy's CG on calcocce / calcoccg,
    minimization.py:77-97) at the sizes of ``--occ-nbf`` (ndoc = nbf // 10,
    ncwo = 4, nbf5 = nbf / 2; 300 and 600 are the c2 and c3 shapes): on the
    device (ops.OccMinimizer,
    one CUDA graph per minimisation) and as the host form (scipy's CG over
    the compiled host evaluation).  J_MO, K_MO, H_core come from the FP64
    device computeJKH_MO at seeded synthetic orbitals; gamma starts from the
    reference's softmax guess.  Device: CUDA events over --steps
    minimisations after --warmup (``e2e_ms`` adds the copy of gamma, n,
    C^J, C^K to the host and the synchronisation, as the solver makes it);
    host: wall clock, best of 3."""
    import scipy.optimize
    import torch

    from pynof_gb300 import nof, ops, synthetic

    torch.cuda.set_device(0)
    sizes = {}
    for nbf in (int(x) for x in args.occ_nbf.split(",")):
        name, st = f"nbf={nbf}", synthetic.Structure.for_nbf(nbf)
        b, C, H, _ = synthetic.make_inputs(st, seed=0)
        db = ops.to_device(b)
        del b
        J, K, Hc = ops.jkh_mo_ri(ops.to_device(C), ops.to_device(H), db, st.nbf5)
        del db
        g0 = nof.gamma_guess_softmax(st)
        dg = ops.to_device(g0)
        om = ops.OccMinimizer(st.nbf5, st.no1, st.ndoc, st.ncwo)
        for _ in range(args.warmup):
            om.minimize(dg, J, K, Hc)
        torch.cuda.synchronize()
        stream = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            om.minimize(dg, J, K, Hc)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        res = om.result.cpu().numpy()
        t = []
        for _ in range(3):
            t0 = time.perf_counter()
            outs = om.minimize(dg, J, K, Hc)
            [o.cpu() for o in (outs[0], outs[1], outs[2], outs[3], outs[4])]
            t.append(time.perf_counter() - t0)
        fn = nof.OccFunction(J.cpu().numpy(), K.cpu().numpy(), Hc.cpu().numpy(), st)
        th = []
        for _ in range(3):
            t0 = time.perf_counter()
            ref = scipy.optimize.minimize(fn, g0, jac=True, method="CG")
            th.append(time.perf_counter() - t0)
        sizes[name] = {"nbf5": st.nbf5, "nv": st.nv,
                       "device": {"ms": ms, "iterations": int(res[1]), "evaluations": int(res[2]),
                                  "us_per_evaluation": 1e3 * ms / res[2], "e2e_ms": 1e3 * min(t),
                                  "E": float(res[0]), "success": bool(res[3] == 1.0)},
                       "host_scipy": {"ms": 1e3 * min(th), "iterations": int(ref.nit), "evaluations": int(ref.nfev),
                                      "E": float(ref.fun)},
                       "speedup_e2e": min(th) / min(t), "E_rel_diff": abs(res[0] - ref.fun) / abs(ref.fun)}
        om.close()
    line = {"mode": "occ", "metric": "occupation minimisation time (occoptr, scipy's CG on calcocce/calcoccg)",
            "unit": "ms", "data": "synthetic (J_MO, K_MO, H_core from the FP64 device computeJKH_MO)",
            "config": {"steps": args.steps, "warmup": args.warmup, "gtol": 1e-5}, "sizes": sizes}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.mode == "batch":
        run_batch(args)
    elif args.mode == "serve":
        run_serve(args)
    elif args.mode == "precision":
        run_precision(args)
    elif args.mode == "mo":
        run_mo(args)
    elif args.mode == "hostlink":
        run_hostlink(args)
    elif args.mode == "occ":
        run_occ(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
