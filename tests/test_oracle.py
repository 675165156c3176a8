"""The CPU oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the compiled reference), and against the
live reference library where its sources are present."""
import numpy as np
import pytest

from marx_gb300 import workloads as W
from marx_gb300.photons import predraw_variates, NUM_U, NUM_N
from oracle.bindings import Oracle, Reference, reference_available

from helpers import load_trace_fixture, compare

NAMES = list(W.PLAIN)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_fixture_bit_exact(name):
    w, ph, U, N, z = load_trace_fixture(name)
    o = Oracle(w.cfg)
    q = ph.copy()
    assert o.trace(q, U=U, N=N, threads=2) == 0
    r = compare(q, z)
    assert r["dx"] == 0.0 and r["dp"] == 0.0, r
    assert all(v == 0 for k, v in r.items() if k not in ("dx", "dp")), r


@pytest.mark.parametrize("name", NAMES)
def test_fixture_exercises_the_path(name):
    """The fixtures cover detections, absorptions and (for HETG) many orders."""
    _, _, _, _, z = load_trace_fixture(name)
    good = (z["flags"] & 0xFF) == 0
    assert 0.03 < good.mean() < 0.6
    assert np.any(z["flags"] & 0x02)                 # unreflected photons
    assert np.unique(z["ccd_num"][good]).size >= 1
    if name == "plain_hetg":
        assert np.unique(z["order"][good]).size >= 3
    if name == "plain_scatter":
        assert z["used"][:, 2].max() == 12            # every mirror slot drawn (blur, WFold)


@pytest.mark.skipif(not reference_available(), reason="reference sources not present")
@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_live_reference(name):
    w = W.PLAIN[name](parity=True)
    n = 4000
    ph = w.photons(n, seed=12345)
    U, N = predraw_variates(n, seed=777)
    ref_q, used, bad = Reference(w.cfg).trace_slots(ph, U, N)
    assert bad == 0
    q = ph.copy()
    Oracle(w.cfg).trace(q, U=U, N=N, threads=2)
    r = compare(q, ref_q)
    assert r["dx"] == 0.0 and r["dp"] == 0.0 and all(v == 0 for k, v in r.items() if k not in ("dx", "dp")), r


@pytest.mark.skipif(not reference_available(), reason="reference sources not present")
def test_oracle_chip_geometry_matches_reference():
    for det in (1, 2):
        w = W.plain_onaxis(parity=True)
        w.cfg.detector = det
        g1 = Reference(w.cfg).detector_geometry()
        g2 = Oracle(w.cfg).detector_geometry()
        assert g1.shape == g2.shape and np.array_equal(g1, g2)


def test_oracle_threads_do_not_change_results():
    w = W.plain_hetg(parity=True)
    ph = w.photons(3000, seed=5)
    o = Oracle(w.cfg)
    a, b = ph.copy(), ph.copy()
    o.trace(a, seed=9, threads=1)
    o.trace(b, seed=9, threads=4)
    r = compare(a, b)
    assert r["dx"] == 0 and all(v == 0 for k, v in r.items() if k not in ("dx", "dp"))


def test_philox_variates_are_uniform_and_normal():
    o = Oracle(W.plain_onaxis().cfg)
    u = np.array([o.philox_uniform(42, t, k) for t in range(2000) for k in range(NUM_U)])
    g = np.array([o.philox_normal(42, t, k) for t in range(2000) for k in range(NUM_N)])
    assert 0.0 <= u.min() and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.01 and abs(u.var() - 1 / 12) < 0.005
    assert abs(g.mean()) < 0.03 and abs(g.std() - 1.0) < 0.03
    assert o.philox_uniform(42, 7, 3) == o.philox_uniform(42, 7, 3)
    assert o.philox_uniform(42, 7, 3) != o.philox_uniform(43, 7, 3)


def test_variate_overrun_is_flagged_not_silent():
    """With one open shutter quadrant the aperture loop can need more
    uniforms than the mirror's slot window; such photons are flagged."""
    w = W.plain_onaxis(parity=True)
    for i in range(4):
        w.cfg.shutters[i] = 0x1
    ph = w.photons(4000)
    U, N = predraw_variates(4000, seed=3)
    q = ph.copy()
    nbad = Oracle(w.cfg).trace(q, U=U, N=N)
    assert nbad > 0
    assert np.count_nonzero(q.flags & 0x10000) == nbad


def test_flop_count_is_positive_and_ordered():
    counts = {}
    for name in NAMES:
        w = W.PLAIN[name]()
        ph = w.photons(2000, seed=1)
        ops, n = Oracle(w.cfg).count_flops(ph, seed=3)
        counts[name] = ops / n
    assert 50 < counts["plain_onaxis"] < counts["plain_scatter"]
    assert counts["plain_hetg"] > 0
