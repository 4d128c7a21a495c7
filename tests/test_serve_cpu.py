"""Admission, continuous batching and failure isolation of the serving loop,
with a fake solve on the host (no GPU): requests that raise fail alone,
requests above the HBM budget are rejected, the slot and budget limits hold."""
import threading
import time

import pytest

from pynof_gb300 import serve


def make_server(budget, slots, fail=(), delay=0.05):
    srv = serve.Server(hbm_budget=budget, slots=slots, device="cpu")
    lock = threading.Lock()
    live = {"now": 0, "peak": 0}

    def fake(req):
        with lock:
            live["now"] += 1
            live["peak"] = max(live["peak"], live["now"])
        try:
            time.sleep(delay)
            if req.rid in fail:
                raise RuntimeError("injected failure")
            return -float(req.nbf), True, 3
        finally:
            with lock:
                live["now"] -= 1

    srv.solve_fn = fake
    return srv, live


def test_slots_and_failures():
    reqs = [serve.Request(i, 24 + i, 1000 + i, 0.0) for i in range(10)]
    srv, live = make_server(1e12, 3, fail=(4,))
    rep = srv.run(reqs, realtime=False)
    assert rep["completed"] == 9 and rep["failed"] == 1
    assert srv.errors[0][0] == 4 and "injected" in srv.errors[0][1]
    assert 1 < live["peak"] <= 3 and rep["peak_active"] <= 3
    assert sorted(r.rid for r in srv.results) == [i for i in range(10) if i != 4]
    assert srv.reserved == 0 and srv.active == 0


def test_budget_admission():
    small = serve.reservation_bytes(serve.synthetic.Structure.for_nbf(30), "mixed", 6)
    big = serve.reservation_bytes(serve.synthetic.Structure.for_nbf(200), "mixed", 6)
    assert big > 2 * small
    # room for two small requests at a time, never for the big one
    reqs = [serve.Request(i, 30, 1000 + i, 0.0) for i in range(5)] + [serve.Request(9, 200, 9, 0.0)]
    srv, live = make_server(2.5 * small, 8)
    rep = srv.run(reqs, realtime=False)
    assert rep["completed"] == 5 and rep["failed"] == 1 and srv.errors[0][0] == 9
    assert live["peak"] == 2 and rep["peak_reserved_gb"] * 1e9 <= 2.5 * small


def test_poisson_stream_shape():
    reqs = serve.poisson_stream(200, rate=50.0, nbf_lo=24, nbf_hi=600, seed=3)
    sizes = [r.nbf for r in reqs]
    assert min(sizes) >= 24 and max(sizes) <= 600
    gaps = [b.arrival - a.arrival for a, b in zip(reqs, reqs[1:])]
    assert all(g >= 0 for g in gaps)
    assert 0.5 / 50 < sum(gaps) / len(gaps) < 2.0 / 50
