"""The ACIS response on the GPU (the pass after the trace) against the
reference's own ACIS detector reading the same synthetic FEF and
contamination files: with DetIdeal = yes the FEF pulse heights, with
DetIdeal = no also the CALDB QE x contamination acceptance.  Per-photon
fixtures with pre-drawn variates (every column exact, PHA and PI included)
and seeded statistics with the reference's generator (PHA and PI histograms
by chi-square, detected and streaked fractions)."""
import os

import numpy as np
import pytest

from marx_gb300 import workloads as W
from marx_gb300.caldb.pack import DEFAULT_PACK, pack_with_fef
from marx_gb300.photons import PhotonList

from helpers import GOLDEN, pad_slots, assert_parity
from test_statistics_gpu import chi2_p

pytestmark = pytest.mark.gpu
FEF_FILE = os.path.join(GOLDEN, "acis_fef_synthetic.fits")
CONTAM_FILE = os.path.join(GOLDEN, "acis_contam_synthetic.fits")
# fixture: (workload, DetIdeal)
CASES = {"fef_acis_i": ("plain_scatter", 1), "fef_hetg_s": ("plain_hetg", 1),
         "qe_acis_i": ("plain_scatter", 0), "qe_hetg_s": ("plain_hetg", 0)}


@pytest.fixture(scope="module")
def fef_pack(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("fef") / "fef.mxpack")
    pack_with_fef(DEFAULT_PACK, FEF_FILE, out, contam_path=CONTAM_FILE)
    return out


def case_config(name):
    base, ideal = CASES[name]
    cfg = W.ALL[base](parity=True).cfg
    cfg.det_ideal = ideal
    return cfg


def engine(cfg, pack, mode=0):
    from marx_gb300._native import Engine
    e = Engine(cfg, pack=pack)
    e.set_mode(mode)
    return e


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("name", list(CASES))
def test_fef_matches_reference_fixture(cuda, fef_pack, name, mode):
    import torch
    from marx_gb300._native import DevicePhotons
    z = np.load(os.path.join(GOLDEN, f"trace_{name}.npz"))
    ph = PhotonList.from_inputs(z["energy"], z["p_in"], z["arrival_time"])
    U, N = pad_slots(z["U"], z["N"])
    eng = engine(case_config(name), fef_pack, mode)
    d = DevicePhotons.from_host(ph)
    eng.trace(d, U=torch.from_numpy(U).cuda(), N=torch.from_numpy(N).cuda())
    torch.cuda.synchronize()
    q = d.to_host()
    assert_parity(q, z, f"{name} mode {mode}")
    on = z["ccd_num"] >= 0
    assert np.array_equal(q.pulse_height[on], z["pulse_height"][on]), name
    assert np.array_equal(q.pi[on], z["pi"][on]), name
    assert (z["pulse_height"][on] > 0).sum() > 40


def test_fef_host_entry_and_launch_count(cuda, fef_pack):
    z = np.load(os.path.join(GOLDEN, "trace_fef_acis_i.npz"))
    ph = PhotonList.from_inputs(z["energy"], z["p_in"], z["arrival_time"])
    U, N = pad_slots(z["U"], z["N"])
    eng = engine(case_config("fef_acis_i"), fef_pack)
    l0 = eng.launch_count()
    eng.trace_host(ph, U=U, N=N)
    assert eng.launch_count() - l0 == 2                  # the fused trace, then the FEF pass
    on = z["ccd_num"] >= 0
    assert np.array_equal(ph.pulse_height[on], z["pulse_height"][on])
    assert np.array_equal(ph.pi[on], z["pi"][on])


@pytest.mark.parametrize("name", list(CASES))
def test_fef_statistics(cuda, fef_pack, name):
    import torch
    from marx_gb300._native import DevicePhotons
    ref = np.load(os.path.join(GOLDEN, f"stats_{name}.npz"))
    w = W.ALL[CASES[name][0]](parity=True)
    eng = engine(case_config(name), fef_pack)
    d = DevicePhotons.from_host(w.photons(200_000, seed=w.seed + 14))
    eng.trace(d, seed=77)
    torch.cuda.synchronize()
    q = d.to_host()
    good = (q.flags & 0xFF) == 0
    hit = q.ccd_num >= 0
    assert eng.overrun_count() == 0
    n_ref, n_gpu = int(ref["on_chip"]), int(hit.sum())
    # FEF-detected fraction of the photons on a chip, and streaked fraction, within 5 sigma
    for k_ref, k_gpu in ((int(ref["good"]), int(good.sum())), (int(ref["streaked"]), int(((q.flags & 0x200) != 0).sum()))):
        pr, pg = k_ref / n_ref, k_gpu / n_gpu
        sig = np.sqrt(pr * (1 - pr) / n_ref + pg * (1 - pg) / n_gpu) + 1e-12
        assert abs(pr - pg) < 5 * sig, (name, pr, pg)
    pha = np.bincount(np.clip(q.pulse_height[good].astype(int), 0, 1023) // 8, minlength=128)
    assert chi2_p(pha, ref["pha_hist"]) > 1e-4
    pi = np.histogram(q.pi[good], bins=np.linspace(0, 12, 97))[0]
    assert chi2_p(pi, ref["pi_hist"]) > 1e-4
    if CASES[name][1]:       # DetIdeal: every photon on a chip that is not detected failed in the FEF
        assert np.all(q.pulse_height[hit & ~good] == -1) and np.all(q.pi[hit & ~good] == 0)


def test_fef_pipelined_host_entry_equals_device_trace(cuda, fef_pack):
    """With an FEF, the chunked host entry (several streams, the FEF pass per
    chunk) equals the one-pass device trace column for column."""
    import torch
    from marx_gb300._native import DevicePhotons
    w = W.ALL["plain_scatter"]()
    n = (1 << 21) + 777
    ph = w.photons(n, seed=21)
    cfg = w.cfg
    cfg.det_ideal = 0                        # QE and contamination too
    eng = engine(cfg, fef_pack)
    a = ph.copy()
    eng.trace_host(a, seed=4)
    d = DevicePhotons.from_host(ph)
    eng.trace(d, seed=4)
    torch.cuda.synchronize()
    b = d.to_host()
    for k in ("x", "p", "flags", "ccd_num", "y_pixel", "z_pixel", "pulse_height", "pi"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert (a.pulse_height > 0).sum() > n // 20
