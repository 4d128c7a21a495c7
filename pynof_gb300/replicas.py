"""Replica bookkeeping for runs over several GPUs of one node.

The JK build exchanges no data between GPUs: J_i, K_i are independent in the
orbital index i and molecules are independent of each other, so each rank runs
its own replica of the workload (its own b, its own orbitals or molecules).
The only cross-rank steps are the barrier on both sides of the timed region
and the reduction of the timings: the whole-job throughput is the units all
ranks processed divided by the slowest rank's time.

Ranks come from the usual launcher variables (WORLD_SIZE, RANK, LOCAL_RANK,
MASTER_ADDR, MASTER_PORT).  With one rank nothing is initialised.
"""
from __future__ import annotations

import os

import torch
import torch.distributed as dist


class Replicas:
    def __init__(self, backend: str | None = None, device: torch.device | None = None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.device = device if device is not None else torch.device("cpu")
        self.backend = backend or ("nccl" if self.device.type == "cuda" else "gloo")
        self._owns = False
        if self.world > 1 and not dist.is_initialized():
            kw = {"device_id": self.device} if self.backend == "nccl" else {}
            dist.init_process_group(self.backend, **kw)
            self._owns = True

    def _reduce(self, x: float, op) -> float:
        if self.world == 1:
            return float(x)
        dev = self.device if self.backend == "nccl" else torch.device("cpu")
        t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=op)
        return float(t.item())

    def barrier(self) -> None:
        """All ranks here, and (on a GPU) this rank's queued work finished."""
        if self.world > 1:
            dist.barrier()
        if self.device.type == "cuda":
            torch.cuda.synchronize(self.device)

    def max(self, x: float) -> float:
        return self._reduce(x, dist.ReduceOp.MAX)

    def sum(self, x: float) -> float:
        return self._reduce(x, dist.ReduceOp.SUM)

    def throughput(self, units: float, seconds: float) -> tuple[float, float]:
        """(whole-job units/s, slowest rank's seconds) from this rank's share."""
        total = self.sum(units)
        slowest = self.max(seconds)
        return total / slowest, slowest

    def close(self) -> None:
        if self._owns and dist.is_initialized():
            dist.destroy_process_group()
            self._owns = False
