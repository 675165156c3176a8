"""GPU trace against the reference's outputs and the CPU oracle.

Tolerances (the parity contract): positions within 1e-9 mm, directions
within 1e-12, and flags, mirror shell, grating order, chip, pixel and
dither state exact.
"""
import numpy as np
import pytest

from marx_gb300 import workloads as W
from marx_gb300.photons import PhotonList, predraw_variates, BAD_PHOTON_MASK

from helpers import load_trace_fixture, assert_parity, compare

pytestmark = pytest.mark.gpu
NAMES = list(W.PLAIN)
ALL_NAMES = list(W.ALL)        # with the workloads pinned to reference fixtures only


def engine(cfg, mode=0):
    from marx_gb300._native import Engine
    e = Engine(cfg)
    e.set_mode(mode)
    return e

MODES = {"fused": 1, "wavefront": 2}


def device_trace(eng, ph, U=None, N=None, seed=0, stages=15):
    import torch
    from marx_gb300._native import DevicePhotons
    d = DevicePhotons.from_host(ph)
    Ud = torch.from_numpy(U).cuda() if U is not None else None
    Nd = torch.from_numpy(N).cuda() if N is not None else None
    eng.trace(d, stages=stages, U=Ud, N=Nd, seed=seed)
    torch.cuda.synchronize()
    return d.to_host()


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("name", ALL_NAMES)
def test_gpu_matches_reference_fixture(cuda, name, mode):
    w, ph, U, N, z = load_trace_fixture(name)
    eng = engine(w.cfg, MODES[mode])
    q = device_trace(eng, ph, U, N)
    assert_parity(q, z, f"{name} device buffers {mode}")
    assert eng.overrun_count() == 0


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("name", ALL_NAMES)
def test_gpu_host_entry_matches_reference_fixture(cuda, name, mode):
    w, ph, U, N, z = load_trace_fixture(name)
    eng = engine(w.cfg, MODES[mode])
    q = ph.copy()
    eng.trace_host(q, U=U, N=N)
    assert_parity(q, z, f"{name} host buffers")


@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_oracle_philox(cuda, name):
    from oracle.bindings import Oracle
    w = W.PLAIN[name]()
    ph = w.photons(200_000, seed=4242)
    a = ph.copy()
    Oracle(w.cfg).trace(a, seed=31337)
    q = device_trace(engine(w.cfg), ph, seed=31337)
    assert_parity(q, a, f"{name} philox", pixel_ulps=1)


@pytest.mark.parametrize("name", ALL_NAMES)
def test_wavefront_equals_fused(cuda, name):
    w = W.ALL[name]()
    ph = w.photons(100_000, seed=77)
    a = device_trace(engine(w.cfg, MODES["fused"]), ph, seed=3)
    b = device_trace(engine(w.cfg, MODES["wavefront"]), ph, seed=3)
    assert_parity(b, a, f"{name} wavefront vs fused")


@pytest.mark.parametrize("name", ALL_NAMES)
def test_split_stages_equal_fused(cuda, name):
    w, ph, U, N, z = load_trace_fixture(name)
    eng = engine(w.cfg, MODES["fused"])
    fused = device_trace(eng, ph, U, N)
    import torch
    from marx_gb300._native import DevicePhotons
    d = DevicePhotons.from_host(ph)
    Ud, Nd = torch.from_numpy(U).cuda(), torch.from_numpy(N).cuda()
    for st in (1, 2, 4, 8):
        eng.trace(d, stages=st, U=Ud, N=Nd)
    torch.cuda.synchronize()
    r = compare(d.to_host(), fused)
    assert r["dx"] == 0 and r["dp"] == 0 and all(v == 0 for k, v in r.items() if k not in ("dx", "dp")), r


@pytest.mark.parametrize("mode", list(MODES))
def test_empty_single_and_ragged_lists(cuda, mode):
    from oracle.bindings import Oracle
    w = W.plain_hetg()
    eng = engine(w.cfg, MODES[mode])
    o = Oracle(w.cfg)
    for n in (0, 1, 31, 257, 4099):
        ph = w.photons(n, seed=n + 1)
        a = ph.copy()
        o.trace(a, seed=5)
        q = device_trace(eng, ph, seed=5)
        if n:
            assert_parity(q, a, f"n={n}")
        q2 = ph.copy()
        eng.trace_host(q2, seed=5)
        if n:
            assert_parity(q2, a, f"host n={n}")


@pytest.mark.parametrize("mode", list(MODES))
def test_bad_photons_are_left_untouched(cuda, mode):
    w = W.plain_scatter()
    ph = w.photons(10_000, seed=8)
    ph.flags[::3] = 0x08       # already missed: every stage skips them
    q = device_trace(engine(w.cfg, MODES[mode]), ph, seed=1, stages=14)
    pre = (ph.flags & BAD_PHOTON_MASK) != 0
    assert np.array_equal(q.p[:, pre], ph.p[:, pre])
    assert np.array_equal(q.x[:, pre], ph.x[:, pre])
    assert np.array_equal(q.flags[pre], ph.flags[pre])


def test_out_of_table_energies_match_oracle(cuda):
    from oracle.bindings import Oracle
    w = W.plain_hetg()
    ph = w.photons(5000, seed=2)
    ph.energy[:] = np.linspace(0.05, 12.0, ph.n)   # beyond both ends of every table
    a = ph.copy()
    Oracle(w.cfg).trace(a, seed=11)
    q = device_trace(engine(w.cfg), ph, seed=11)
    assert_parity(q, a, "edge energies")


@pytest.mark.parametrize("mode", list(MODES))
def test_variate_overrun_matches_oracle(cuda, mode):
    from oracle.bindings import Oracle
    w = W.plain_onaxis(parity=True)
    for i in range(4):
        w.cfg.shutters[i] = 0x1
    ph = w.photons(4000)
    U, N = predraw_variates(4000, seed=3)
    a = ph.copy()
    nbad = Oracle(w.cfg).trace(a, U=U, N=N)
    eng = engine(w.cfg, MODES[mode])
    q = device_trace(eng, ph, U, N)
    assert nbad > 0 and eng.overrun_count() == nbad
    assert_parity(q, a, f"overrun {mode}")


def test_compaction_matches_prune(cuda):
    import torch
    w = W.plain_scatter()
    eng = engine(w.cfg)
    for n in (1, 1000, 4096, 4097, 300_001):
        flags = np.random.default_rng(n).integers(0, 4, n).astype(np.uint32) * 0x04
        t = torch.from_numpy(flags.view(np.int32)).cuda()
        idx = eng.compact(t).cpu().numpy()
        assert np.array_equal(idx, np.nonzero((flags & BAD_PHOTON_MASK) == 0)[0])


def test_launch_count_tracks_kernels(cuda):
    w = W.plain_onaxis()
    eng = engine(w.cfg, MODES["fused"])
    before = eng.launch_count()
    device_trace(eng, w.photons(1000))
    assert eng.launch_count() == before + 1
    eng.set_mode(MODES["wavefront"])
    device_trace(eng, w.photons(1000))
    assert eng.launch_count() == before + 1 + 4   # phases A, T, B and C


@pytest.mark.parametrize("slots,n", [(False, (1 << 21) + 12345), (True, (1 << 21) + 12345), (False, (1 << 19) + 333)])
def test_pipelined_host_entry_equals_device_trace(cuda, slots, n):
    """mx_trace_host on a list large enough to be cut into chunks
    (copies overlapping the traces of other chunks; 7 chunks at these
    sizes, 19 from 2^23 photons, which the 2e7-photon HETG test in
    test_full_size_gpu.py takes): every column equals the one-pass device
    trace of the same photons, with Philox draws and with pre-drawn
    variates (packed per chunk)."""
    w = W.ALL["plain_scatter"]()
    ph = w.photons(n, seed=9)
    U, N = predraw_variates(n, 3) if slots else (None, None)
    eng = engine(w.cfg)
    a = ph.copy()
    eng.trace_host(a, U=U, N=N, seed=5)
    b = device_trace(eng, ph, U, N, seed=5)
    for k in ("x", "p", "flags", "mirror_shell", "order", "ccd_num", "y_pixel", "z_pixel", "dither_state"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert int(((a.flags & BAD_PHOTON_MASK) == 0).sum()) > n // 10


def _take(ph, idx):
    """The photons idx of a list (every column, tags included)."""
    from marx_gb300.photons import COLUMNS
    q = ph.copy()
    for k in COLUMNS:
        setattr(q, k, np.ascontiguousarray(getattr(ph, k)[..., idx]))
    q.n = len(idx)
    return q


def test_split_device_trace_is_independent_of_the_partition(cuda):
    """From 2^18 photons a device trace runs in two parts at once on two
    streams.  Photons are independent and draw by tag, so the list traced
    reversed (split at another photon) gives the reversed result, and its
    first 2^17 photons traced alone (one pass) give the same columns."""
    n = (1 << 19) + 4321
    w = W.ALL["plain_scatter"]()
    ph = w.photons(n, seed=12)
    eng = engine(w.cfg)
    a = device_trace(eng, ph, seed=8)
    rev = np.arange(n)[::-1]
    b = device_trace(eng, _take(ph, rev), seed=8)
    head = np.arange(1 << 17)
    c = device_trace(eng, _take(ph, head), seed=8)
    for k in ("x", "p", "flags", "mirror_shell", "order", "ccd_num", "y_pixel", "z_pixel", "dither_state"):
        va = getattr(a, k)
        assert np.array_equal(va, getattr(b, k)[..., rev]), k
        assert np.array_equal(va[..., head], getattr(c, k)), k
    assert int(((a.flags & BAD_PHOTON_MASK) == 0).sum()) > n // 10


def test_pipelined_host_entry_without_tags(cuda):
    """A list without a tag column draws photon i with generator counter i
    (its index in the list): each chunk of the pipelined host entry counts
    from its first photon's index in the whole list, so the trace equals
    the one-pass device trace of the same photons tagged 0 .. n - 1."""
    n = (1 << 20) + 777
    w = W.ALL["plain_scatter"]()
    ph = w.photons(n, seed=10)
    ph.tag = np.arange(n, dtype=np.uint32)
    eng = engine(w.cfg)
    a = ph.copy()
    a.tag = None
    eng.trace_host(a, seed=6)
    b = device_trace(eng, ph, seed=6)
    for k in ("x", "p", "flags", "mirror_shell", "order", "ccd_num", "y_pixel", "z_pixel", "dither_state"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert int(((a.flags & BAD_PHOTON_MASK) == 0).sum()) > n // 10
