"""The trace at the configurations' full sizes against the CPU oracle.

The on-axis configuration (1e6 photons), the scattered, dithered one
(1e7) and the HETG one (2e7, ACIS-S) are traced on the GPU with Philox
draws and compared photon by photon with the oracle's trace of the same
photons and draws, under the parity contract (positions within 1e-9 mm,
directions within 1e-12; flags, shell, order, chip, pixels and dither state
exact).  At these sizes the index arithmetic, the growth of the wavefront
queues from a smaller list and, through mx_trace_host, the chunk seams of
the pipelined host entry are all exercised against an independent result.
The oracle rounds without fused multiply-add, the GPU with it, so FP64
positions agree to a few 1e-10 mm; about one detected photon in a million
then has a single-precision pixel one float step away from the oracle's
(a rounding boundary between the two positions), with the whole pixel
equal.
"""
import numpy as np
import pytest

from marx_gb300 import workloads as W
from marx_gb300.photons import BAD_PHOTON_MASK

from helpers import assert_parity

pytestmark = pytest.mark.gpu


def _oracle(w, ph, seed):
    from oracle.bindings import Oracle
    a = ph.copy()
    Oracle(w.cfg).trace(a, seed=seed)
    return a


def _device(eng, ph, seed):
    import torch
    from marx_gb300._native import DevicePhotons
    d = DevicePhotons.from_host(ph)
    eng.trace(d, seed=seed)
    torch.cuda.synchronize()
    q = d.to_host()
    del d
    torch.cuda.empty_cache()
    return q


@pytest.mark.parametrize("name", ["plain_onaxis", "plain_scatter"])
def test_full_size_device_trace_matches_oracle(cuda, name):
    from marx_gb300._native import Engine
    w = W.PLAIN[name]()
    ph = w.photons()
    assert ph.n == w.n
    q = _device(Engine(w.cfg), ph, seed=2718)
    assert_parity(q, _oracle(w, ph, 2718), f"{name} at {w.n} photons", pixel_ulps=1)
    assert int(((q.flags & BAD_PHOTON_MASK) == 0).sum()) > w.n // 20


def test_full_size_hetg_device_and_host_entries_match_oracle(cuda):
    """2e7 HETG photons: the device entry (queues grown on the same context
    from a 1e6-photon trace first) and the host entry (16 chunks on three
    streams) against the oracle."""
    from marx_gb300._native import Engine
    w = W.plain_hetg()
    ph = w.photons()
    assert ph.n == 20_000_000
    eng = Engine(w.cfg)
    small = w.photons(1_000_000, seed=5)
    assert_parity(_device(eng, small, 99), _oracle(w, small, 99), "hetg 1e6 before growth", pixel_ulps=1)
    ref = _oracle(w, ph, 1414)
    q = _device(eng, ph, 1414)
    assert_parity(q, ref, "hetg 2e7 device entry", pixel_ulps=1)
    del q
    h = ph.copy()
    eng.trace_host(h, seed=1414)
    assert_parity(h, ref, "hetg 2e7 host entry (chunked)", pixel_ulps=1)
    det = (h.flags & BAD_PHOTON_MASK) == 0
    assert det.sum() > 1_000_000
    # every order -3..3 reaches the ACIS-S, and both signs of each
    orders = np.unique(h.order[det])
    assert set(range(-3, 4)) <= set(orders.tolist())
