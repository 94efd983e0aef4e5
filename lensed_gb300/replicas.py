"""Replica bookkeeping for multi-GPU runs (one process per GPU).

The likelihood path shards over independent candidates: each rank evaluates
its own batch on its own GPU and no data crosses ranks.  What the ranks share
is bookkeeping, done on the host with ``torch.distributed``:

* ``init``: process group from RANK / WORLD_SIZE / MASTER_* (nccl on GPUs,
  gloo on CPUs), with a timeout so that a rank that died makes the others
  fail instead of hang;
* ``max_over_ranks``: the slowest rank's time (the job's time);
* ``aggregate``: whole-job throughput = units of all ranks / that time;
* ``Heartbeat``: a store-based liveness check between steps, so a rank that
  left is noticed before the next launch.
"""
from __future__ import annotations

import datetime
import os
import time
from typing import Optional, Tuple


def env() -> Tuple[int, int, int]:
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: Optional[str] = None, timeout_s: float = 300.0):
    """Initialise the process group when WORLD_SIZE > 1; returns (rank,
    world, local_rank, dist-or-None)."""
    rank, world, local = env()
    if world <= 1:
        return rank, world, local, None
    import torch.distributed as dist

    if backend is None:
        import torch

        backend = "nccl" if torch.cuda.is_available() else "gloo"
    dist.init_process_group(backend, timeout=datetime.timedelta(seconds=timeout_s))
    return rank, world, local, dist


def candidate_seed(rank: int, base: int = 1) -> int:
    """Each rank draws its own candidates (weak scaling)."""
    return base + rank


def max_over_ranks(value: float, dist=None, device: str = "cpu") -> float:
    if dist is None:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate(units_per_rank: float, max_seconds: float, world: int) -> float:
    """Whole-job throughput: every rank processed units_per_rank units; the
    job took as long as its slowest rank."""
    return world * units_per_rank / max_seconds


class Heartbeat:
    """Liveness check through the process group's store: each rank marks
    each step it reaches; ``missing(step)`` lists ranks that have not marked
    it within the timeout (a rank that exited between steps)."""

    def __init__(self, store, rank: int, world: int, timeout_s: float = 10.0):
        self.store, self.rank, self.world, self.timeout = store, rank, world, timeout_s

    def beat(self, step: int) -> None:
        self.store.set(f"lg_hb/{step}/{self.rank}", str(time.time()))

    def missing(self, step: int):
        out = []
        for r in range(self.world):
            if r == self.rank:
                continue
            try:
                self.store.wait([f"lg_hb/{step}/{r}"], datetime.timedelta(seconds=self.timeout))
            except Exception:
                out.append(r)
        return out
