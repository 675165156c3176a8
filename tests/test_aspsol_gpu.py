"""DitherModel = FILE on the GPU against the reference's own dither and
detector stages reading the same synthetic aspect solution
(tests/golden/aspsol_synthetic.fits): per-photon fixtures with pre-drawn
variates, every column exact (the sky and detector parts of the dither
state included) and positions within the parity tolerance.  The reference
turns one global detector matrix there and back per photon, which leaves it
a rounding away from the identity; the engine gives each photon its own
frame, hence the tolerance on positions rather than bit equality."""
import os

import numpy as np
import pytest

from marx_gb300 import workloads as W
from marx_gb300.aspsol import apply_to_config, read_aspsol
from marx_gb300.photons import PhotonList

from helpers import GOLDEN, pad_slots, assert_parity

pytestmark = pytest.mark.gpu
ASPSOL_FILE = os.path.join(GOLDEN, "aspsol_synthetic.fits")
CASES = {"aspsol_scatter": "plain_scatter", "aspsol_hrci": "plain_hrci"}
ASPECT_END = 0x80


def engine(name, mode=0, record_only=False, asp=None):
    from marx_gb300._native import Engine
    asp = asp or read_aspsol(ASPSOL_FILE)
    cfg = apply_to_config(W.ALL[CASES[name]](parity=True).cfg, asp)
    e = Engine(cfg)
    e.set_aspect_solution(asp, record_only=record_only)
    e.set_mode(mode)
    return e


def fixture(name):
    z = np.load(os.path.join(GOLDEN, f"trace_{name}.npz"))
    ph = PhotonList.from_inputs(z["energy"], z["p_in"], z["arrival_time"])
    ph.det_dither = np.zeros((3, ph.n), np.float32)
    U, N = pad_slots(z["U"], z["N"])
    return z, ph, U, N


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("name", list(CASES))
def test_file_dither_matches_reference_fixture(cuda, name, mode):
    import torch
    from marx_gb300._native import DevicePhotons
    z, ph, U, N = fixture(name)
    eng = engine(name, mode)
    d = DevicePhotons.from_host(ph)
    eng.trace(d, U=torch.from_numpy(U).cuda(), N=torch.from_numpy(N).cuda())
    torch.cuda.synchronize()
    q = d.to_host()
    assert_parity(q, z, where=f"{name} mode {mode}")
    np.testing.assert_array_equal(q.det_dither, z["det_dither"])
    assert np.abs(z["det_dither"]).max() > 1e-3 and not (q.flags & ASPECT_END).any()


def test_host_entry_carries_the_detector_dither(cuda):
    """mx_trace_host with the det_dither column: the same photons as the
    device entry, the column copied back."""
    z, ph, U, N = fixture("aspsol_scatter")
    eng = engine("aspsol_scatter")
    a = ph.copy()
    eng.trace_host(a, U=U, N=N)
    assert_parity(a, z, where="host entry")
    np.testing.assert_array_equal(a.det_dither, z["det_dither"])


def test_photons_past_the_last_row_are_flagged(cuda):
    """At or after the last row's time the reference's reader runs off the
    end of the file and drops the photon (and the rest of the batch); the
    engine flags it MX_PHOTON_ASPECT_END and later stages leave it alone."""
    import torch
    from marx_gb300._native import DevicePhotons
    asp = read_aspsol(ASPSOL_FILE)
    last = asp.rows[-1, 0] - asp.tstart
    z, ph, U, N = fixture("aspsol_scatter")
    t = ph.arrival_time.copy()
    ph.arrival_time[:] = np.where(np.arange(ph.n) % 3 == 0, last + np.arange(ph.n) * 1e-3, t)
    ph.arrival_time[1] = last                       # exactly at the last row: past the end as well
    eng = engine("aspsol_scatter")
    d = DevicePhotons.from_host(ph)
    eng.trace(d, U=torch.from_numpy(U).cuda(), N=torch.from_numpy(N).cuda())
    q = d.to_host()
    past = ph.arrival_time >= last
    assert past.sum() > 300
    assert ((q.flags & ASPECT_END) != 0).tolist() == past.tolist()
    assert (q.ccd_num[past] == -1).all() and (q.mirror_shell[past] == 0).all()
    np.testing.assert_array_equal(q.p[:, past], ph.p[:, past])
    keep = ~past
    np.testing.assert_array_equal(q.flags[keep], z["flags"][keep])
    np.testing.assert_array_equal(q.y_pixel[keep], z["y_pixel"][keep])


def test_record_only_keeps_the_direction(cuda):
    """Record only (rays already dithered): the state is the same as with
    the dithering model, the pointing does not move the photon; with no
    aspect blur the dither stage only renormalises p."""
    import torch
    from marx_gb300._native import DevicePhotons
    z, ph, U, N = fixture("aspsol_scatter")
    asp = read_aspsol(ASPSOL_FILE)
    w = W.ALL["plain_scatter"](parity=True)
    cfg = apply_to_config(w.cfg, asp)
    cfg.aspect_blur = 0.0
    from marx_gb300._native import Engine
    eng = Engine(cfg)
    eng.set_aspect_solution(asp, record_only=True)
    d = DevicePhotons.from_host(ph)
    eng.trace(d, stages=1, U=torch.from_numpy(U).cuda(), N=torch.from_numpy(N).cuda())
    q = d.to_host()
    np.testing.assert_array_equal(q.dither_state, z["dither_state"])
    np.testing.assert_array_equal(q.det_dither, z["det_dither"])
    assert np.abs(q.p - ph.p).max() < 1e-15


def test_file_model_needs_the_table(cuda):
    from marx_gb300._native import Engine
    cfg = apply_to_config(W.ALL["plain_scatter"](parity=True).cfg, read_aspsol(ASPSOL_FILE))
    eng = Engine(cfg)
    ph = PhotonList.from_inputs(np.full(4, 1.0), np.tile([[-1.0], [0.0], [0.0]], (1, 4)))
    with pytest.raises(RuntimeError, match="aspect_solution"):
        eng.trace_host(ph)
