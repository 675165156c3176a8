"""Batched form: one persistent launch over many sources against the same
photons traced source by source, and against the CPU oracle."""
import numpy as np
import pytest

from marx_gb300 import batched as B
from marx_gb300.config import copy_config

from helpers import assert_parity

pytestmark = pytest.mark.gpu


def small_batch(eng, nsrc=24, seed=9):
    return B.Batch(eng, B.batched_sources(nsrc=nsrc, seed=seed, nmin=200, nmax=40_000))


def engine():
    from marx_gb300._native import Engine
    return Engine(B.batched_config())


def test_batched_equals_sequential(cuda):
    import torch
    eng = engine()
    b = small_batch(eng)
    b.run(seed=77)
    torch.cuda.synchronize()
    one = b.to_host()
    b.run_sequential(seed=77)
    torch.cuda.synchronize()
    seq = b.to_host()
    assert np.array_equal(one.energy, seq.energy) and np.array_equal(one.tag, seq.tag)
    assert_parity(one, seq, "batched vs sequential")
    assert ((one.flags & 0xFF) == 0).mean() > 0.05


@pytest.mark.parametrize("block,tile", [(64, 32), (192, 128)])
def test_every_launch_shape_gives_the_same_photons(cuda, block, tile):
    """The tuner's search space: other block sizes and tiles change who
    traces which photon, never a photon's result."""
    import torch
    eng = engine()
    b = small_batch(eng, nsrc=12, seed=4)
    b.run(seed=9)
    torch.cuda.synchronize()
    ref = b.to_host()
    b.set_params(block, tile, 1)
    b.run(seed=9)
    torch.cuda.synchronize()
    assert_parity(b.to_host(), ref, f"block {block} tile {tile}")


def test_batched_matches_oracle_per_source(cuda):
    import torch
    from oracle.bindings import Oracle
    eng = engine()
    b = small_batch(eng, nsrc=8, seed=3)
    b.run(seed=5)
    torch.cuda.synchronize()
    q = b.to_host()
    start = b.source_start()
    for s, src in enumerate(b.sources):
        n0, n1 = int(start[s]), int(start[s + 1])
        if n1 == n0:
            continue
        cfg = copy_config(B.batched_config())
        cfg.grating, cfg.detector = src.grating, src.detector
        o = Oracle(cfg)
        # the generated photons, as the oracle would make them
        u = np.array([o.source_uniform(5, t) for t in range(n0, n1)])
        energy = src.energy_min + (src.energy_max - src.energy_min) * u
        assert np.array_equal(q.energy[n0:n1], energy)
        from marx_gb300.photons import PhotonList
        ph = PhotonList.from_inputs(energy, np.tile(np.array(src.p[:])[:, None], (1, n1 - n0)))
        ph.tag[:] = np.arange(n0, n1, dtype=np.uint32)
        o.trace(ph, seed=5)
        part = PhotonList.__new__(PhotonList)
        part.n = n1 - n0
        for k in ("x", "p", "dither_state"):
            setattr(part, k, getattr(q, k)[:, n0:n1])
        for k in ("flags", "mirror_shell", "order", "ccd_num", "y_pixel", "z_pixel"):
            setattr(part, k, getattr(q, k)[n0:n1])
        assert_parity(part, ph, f"source {s}", pixel_ulps=1)


def test_tuner_picks_a_valid_shape_and_remembers_it(cuda):
    eng = engine()
    b = small_batch(eng, nsrc=16, seed=1)
    p = b.tune(trials=1)
    assert p["block"] in (64, 128, 192, 256) and p["tile"] % 32 == 0 and p["blocks_per_sm"] >= 1
    b2 = small_batch(eng, nsrc=16, seed=1)
    assert b2.params() == p
    assert b2.tune(trials=1) == p


def test_seeds_reproduce(cuda):
    import torch
    eng = engine()
    b = small_batch(eng, nsrc=6, seed=2)
    b.run(seed=1); torch.cuda.synchronize(); a = b.to_host()
    b.run(seed=2); torch.cuda.synchronize(); c = b.to_host()
    b.run(seed=1); torch.cuda.synchronize(); d = b.to_host()
    assert not np.array_equal(a.energy, c.energy)
    assert np.array_equal(a.energy, d.energy) and np.array_equal(a.x, d.x) and np.array_equal(a.flags, d.flags)


def test_malformed_source_is_rejected(cuda):
    eng = engine()
    srcs = B.batched_sources(nsrc=2, seed=1)
    srcs[1].detector = 0
    with pytest.raises(RuntimeError):
        B.Batch(eng, srcs)
