"""Batched JK builds: many molecules in grouped tensor-core launches, replayed
from a CUDA graph, with tile configurations chosen by an autotuner.

The autotuner times the tile configurations of the half-transform and J
phases (``gb_jkj_batch_create_mixed``'s ``tiles``) on the actual batch and
caches the fastest per (device, slice count, batch signature) in a JSON file
(``$PYNOF_GB300_CACHE`` or ``~/.cache/pynof_gb300/tiles.json``).
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import threading

import torch

from . import _lib, ops

_c = ctypes


def _ptr_array(values):
    arr = (_c.c_void_p * len(values))(*values)
    return arr


def _int_array(values):
    return (_c.c_int * len(values))(*values)


class BatchJK:
    """J_i, K_i for every molecule of a batch, from one CUDA graph.

    mols: list of (C (CUDA tensor, nbf x nbf), PreparedRI, nbf5)."""

    def __init__(self, mols, tiles=(0, 0), stream=None):
        if not mols:
            raise ValueError("empty batch")
        self.mols = mols
        self.S = mols[0][1].nslices
        if any(m[1].nslices != self.S for m in mols):
            raise ValueError("every molecule of a batch uses the same slice count")
        self.dev = mols[0][1].device
        self.stream = stream or torch.cuda.Stream(self.dev)
        self.nbf = [m[1].nbf for m in mols]
        self.naux = [m[1].naux for m in mols]
        self.nbf5 = [m[2] for m in mols]
        self.J = [torch.empty((p, n, n), dtype=torch.float64, device=self.dev) for n, p in zip(self.nbf, self.nbf5)]
        self.K = [torch.empty_like(j) for j in self.J]
        nb, n5, na = _int_array(self.nbf), _int_array(self.nbf5), _int_array(self.naux)
        ws = _lib.query("gb_jkj_batch_workspace_mixed", len(mols), _c.cast(nb, _c.c_void_p),
                        _c.cast(n5, _c.c_void_p), _c.cast(na, _c.c_void_p), self.S)
        self.ws = torch.empty(max(ws, 256), dtype=torch.uint8, device=self.dev)
        self.tiles = tuple(tiles)
        plan = _c.c_void_p()
        Cs = _ptr_array([m[0].data_ptr() for m in mols])
        preps = _ptr_array([m[1].buf.data_ptr() for m in mols])
        Js = _ptr_array([t.data_ptr() for t in self.J])
        Ks = _ptr_array([t.data_ptr() for t in self.K])
        tl = _int_array(list(self.tiles) + [0])
        _lib.call("gb_jkj_batch_create_mixed", len(mols), _c.cast(Cs, _c.c_void_p), _c.cast(preps, _c.c_void_p),
                  _c.cast(nb, _c.c_void_p), _c.cast(n5, _c.c_void_p), _c.cast(na, _c.c_void_p), self.S,
                  _c.cast(Js, _c.c_void_p), _c.cast(Ks, _c.c_void_p), _c.cast(tl, _c.c_void_p),
                  self.ws.data_ptr(), self.ws.numel(), self.stream.cuda_stream, _c.byref(plan))
        self.plan = plan

    def run(self):
        """Replay the graph on the plan's stream (asynchronous)."""
        _lib.call("gb_batch_launch", self.plan, self.stream.cuda_stream)

    def wait(self):
        """Wait for the replays issued so far; raise GBError if a kernel of
        the batch recorded a timeout or met a non-finite operand."""
        self.stream.synchronize()
        ops.check_device_status()

    def close(self):
        """Destroy the graph once every replay has finished: the outputs and
        the workspace go back to torch's allocator only after that."""
        if self.plan:
            self.stream.synchronize()
            _lib.call("gb_batch_destroy", self.plan)
            self.plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# autotuner
# ---------------------------------------------------------------------------
_cache_lock = threading.Lock()


def cache_path() -> str:
    return os.environ.get("PYNOF_GB300_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "pynof_gb300", "tiles.json"))


def signature(mols) -> str:
    sizes = sorted((m[1].nbf, m[2], m[1].naux) for m in mols)
    return hashlib.sha1(json.dumps(sizes).encode()).hexdigest()[:16]


def _time_plan(plan: BatchJK, reps: int = 3) -> float:
    plan.run()
    plan.stream.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(plan.stream)
        plan.run()
        e1.record(plan.stream)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return best


def autotune(mols, reps: int = 3, use_cache: bool = True, log=None) -> tuple[tuple[int, int], dict]:
    """Fastest (half-transform, J) tile configuration for this batch.

    Coordinate search: the half-transform configuration with J at 0, then the
    J configuration with the best half transform.  Returns (tiles, timings)."""
    dev_name = torch.cuda.get_device_name(mols[0][1].device)
    key = f"{dev_name}|S={mols[0][1].nslices}|{signature(mols)}"
    path = cache_path()
    if use_cache:
        with _cache_lock:
            try:
                with open(path) as f:
                    cached = json.load(f).get(key)
                if cached:
                    return tuple(cached["tiles"]), {"cached": True, **cached}
            except (OSError, ValueError):
                pass
    timings = {}

    def measure(t):
        plan = BatchJK(mols, tiles=t)
        try:
            timings[str(t)] = _time_plan(plan, reps)
        finally:
            plan.close()
        if log:
            log(f"tiles {t}: {timings[str(t)] * 1e3:.2f} ms")
        return timings[str(t)]

    best_t = min(range(4), key=lambda tc: measure((tc, 0)))
    best_j = min(range(4), key=lambda jc: timings.get(str((best_t, jc))) or measure((best_t, jc)))
    tiles = (best_t, best_j)
    if use_cache:
        with _cache_lock:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            try:
                with open(path) as f:
                    data = json.load(f)
            except (OSError, ValueError):
                data = {}
            data[key] = {"tiles": list(tiles), "seconds": timings[str(tiles)]}
            with open(path, "w") as f:
                json.dump(data, f, indent=1)
    return tiles, {"cached": False, "timings": timings}
