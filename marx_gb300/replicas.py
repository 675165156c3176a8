"""One process per GPU, each tracing its own photons: the photon list
shards by rank with no exchange on the data path (photons are independent;
MARX itself has no collective).  Used by bench.py under torchrun.

rank_photons  the seeded inputs of one rank, tagged rank * n .. rank * n + n - 1
              so every photon of the job has its own Philox counter
max_over_ranks  the slowest rank's time (the job's time)
"""
from __future__ import annotations

import numpy as np


def rank_photons(workload, n: int, rank: int):
    if (rank + 1) * n > 1 << 32:
        raise ValueError(f"rank {rank} x {n} photons: tags beyond 2^32 would repeat another photon's draws")
    ph = workload.photons(n, seed=workload.seed + rank)
    ph.tag[:] = np.arange(n, dtype=np.uint64).astype(np.uint32) + np.uint32(rank * n)
    return ph


def max_over_ranks(v: float, world: int, device: str = "cuda") -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
