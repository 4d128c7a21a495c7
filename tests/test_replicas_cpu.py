"""Replica timing reduction over two gloo ranks on the CPU (the N>1 bench path)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from pynof_gb300.replicas import Replicas

    r = Replicas(backend="gloo")
    try:
        r.barrier()
        # rank k "built" 10 (k+1) JK builds in 1 + k seconds
        value, slowest = r.throughput(10.0 * (rank + 1), 1.0 + rank)
        q.put((rank, value, slowest, r.max(rank), r.sum(1.0)))
        r.barrier()
    finally:
        r.close()


@pytest.mark.timeout(120)
def test_two_rank_throughput_is_total_over_slowest():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(k, world, port, q)) for k in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=90) for _ in range(world))
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    for rank, value, slowest, mx, sm in out:
        assert slowest == 2.0
        assert value == pytest.approx(30.0 / 2.0)
        assert mx == world - 1
        assert sm == float(world)


def test_single_rank_needs_no_process_group(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from pynof_gb300.replicas import Replicas

    r = Replicas()
    assert r.world == 1
    assert r.throughput(7.0, 2.0) == (3.5, 2.0)
    r.barrier()
    r.close()
