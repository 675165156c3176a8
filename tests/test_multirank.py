"""The multi-GPU path's host logic on two gloo ranks (CPU): each rank traces
its own shard (rank_photons) with the CPU oracle; the gathered shards equal
one process tracing every shard, tags never collide, and the job time is
the slowest rank's (max_over_ranks)."""
import os
import socket

import numpy as np
import pytest

from marx_gb300 import workloads as W
from marx_gb300.replicas import rank_photons, max_over_ranks

N = 3000


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    from oracle.bindings import Oracle
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = W.plain_scatter()
        ph = rank_photons(w, N, rank)
        Oracle(w.cfg).trace(ph, seed=17)
        cols = torch.from_numpy(np.concatenate([ph.x.ravel(), ph.p.ravel(), ph.flags.astype(np.float64),
                                                ph.tag.astype(np.float64), ph.ccd_num.astype(np.float64)]))
        gathered = [torch.zeros_like(cols) for _ in range(world)]
        dist.all_gather(gathered, cols)
        t = max_over_ranks(1.0 + rank, world, device="cpu")
        if rank == 0:
            np.save(out, np.stack([g.numpy() for g in gathered] + [np.full_like(cols.numpy(), t)]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_equal_one_process(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from oracle.bindings import Oracle
    out = str(tmp_path / "gathered.npy")
    mp.spawn(_rank, args=(2, _port(), out), nprocs=2, join=True)
    g = np.load(out)
    assert g[2][0] == 2.0                      # the slower rank's time
    w = W.plain_scatter()
    tags = set()
    for rank in range(2):
        ph = rank_photons(w, N, rank)
        Oracle(w.cfg).trace(ph, seed=17)
        want = np.concatenate([ph.x.ravel(), ph.p.ravel(), ph.flags.astype(np.float64),
                               ph.tag.astype(np.float64), ph.ccd_num.astype(np.float64)])
        assert np.array_equal(g[rank], want)
        tags |= set(ph.tag.tolist())
    assert len(tags) == 2 * N
