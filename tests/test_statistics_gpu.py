"""Seeded GPU runs (Philox variates) against seeded runs of the reference
with its own generator (fixtures in tests/golden/stats_*.npz): survivor
fractions within binomial error, PSF encircled-energy radii under a
two-sample KS test, order and chip histograms under chi-square."""
import os

import numpy as np
import pytest
from scipy import stats

from marx_gb300 import workloads as W

from helpers import GOLDEN

pytestmark = pytest.mark.gpu
N = 200_000


def run_gpu(name, n=N, seed=99):
    import torch
    from marx_gb300._native import Engine, DevicePhotons
    w = W.ALL[name](parity=True)
    eng = Engine(w.cfg)
    d = DevicePhotons.from_host(w.photons(n, seed=w.seed + 10))
    eng.trace(d, seed=seed)
    torch.cuda.synchronize()
    return w, d.to_host()


def chi2_p(a, b):
    keep = (a + b) > 0
    if keep.sum() < 2:        # a single occupied bin: the shapes agree trivially
        return 1.0
    a, b = a[keep].astype(float), b[keep].astype(float)
    ka, kb = np.sqrt(b.sum() / a.sum()), np.sqrt(a.sum() / b.sum())
    chi2 = np.sum((ka * a - kb * b) ** 2 / (a + b))
    return stats.chi2.sf(chi2, keep.sum() - 1)


@pytest.mark.parametrize("name", list(W.ALL))
def test_survivor_fraction_and_histograms(cuda, name):
    ref = np.load(os.path.join(GOLDEN, f"stats_{name}.npz"))
    w, q = run_gpu(name)
    good = (q.flags & 0xFF) == 0
    f_ref, f_gpu = float(ref["good_fraction"]), good.mean()
    sigma = np.sqrt(f_ref * (1 - f_ref) * (1 / N + 1 / int(ref["n"])))
    assert abs(f_gpu - f_ref) < 5 * sigma, (f_gpu, f_ref)
    ccd = np.bincount(q.ccd_num[good].astype(int) + 1, minlength=11)
    assert chi2_p(ccd, ref["ccd_hist"]) > 1e-4
    if "order_hist" in ref:
        m = (len(ref["order_hist"]) - 1) // 2
        orders = np.bincount(q.order[good].astype(int) + m, minlength=2 * m + 1)
        assert chi2_p(orders, ref["order_hist"]) > 1e-4
    if "pha_hist" in ref:       # HRC pulse heights
        pha = np.bincount(q.pulse_height[good].astype(int) // 16, minlength=40)[:40]
        assert chi2_p(pha, ref["pha_hist"]) > 1e-4
    if "region_hist" in ref:    # HRC-S UV/ion shield regions
        reg = np.bincount(q.detector_region[good].astype(int), minlength=4)
        assert chi2_p(reg, ref["region_hist"]) > 1e-4
    if "fine_hist" in ref:      # LETG fine support grating orders
        fine = np.bincount(q.support_orders[0][good].astype(int) + 9, minlength=19)
        assert chi2_p(fine, ref["fine_hist"]) > 1e-4


@pytest.mark.parametrize("name", ["plain_onaxis", "plain_scatter", "plain_hrci"])
def test_psf_encircled_energy(cuda, name):
    ref = np.load(os.path.join(GOLDEN, f"stats_{name}.npz"))
    w, q = run_gpu(name)
    good = (q.flags & 0xFF) == 0
    y, z = q.x[1][good], q.x[2][good]
    r = np.hypot(y - np.median(y), z - np.median(z))
    ee = np.array([(r <= a).mean() for a in ref["ee_radii"]])
    assert np.max(np.abs(ee - ref["ee"])) < 0.01, (ee, ref["ee"])
    assert stats.ks_2samp(np.sort(r)[:: max(1, len(r) // 5000)], ref["radius_sample"]).pvalue > 1e-3


@pytest.mark.parametrize("name", ["plain_hetg", "plain_letg", "letg_hrcs"])
def test_dispersed_spectra(cuda, name):
    """Dispersed spectra: per grating arm (MEG, HEG; LEG) and order -3..3,
    the detected photons' coordinate along the dispersion direction, from
    1e6 photons on the GPU (Philox) against the reference's own seeded run
    of 1e6 (tests/golden/dispersed_*.npz): chi-square over the reference's
    equal-probability bins, two-sample KS on the values, and the split of
    the detected photons over (arm, order) by chi-square."""
    from helpers import dispersed_groups
    ref = np.load(os.path.join(GOLDEN, f"dispersed_{name}.npz"))
    n = int(ref["n"])
    w, q = run_gpu(name, n=n, seed=4242)
    groups = dispersed_groups(q, w.cfg)
    keys = sorted(groups)
    assert keys == sorted(k[len("count_"):] for k in ref.files if k.startswith("count_"))
    counts = np.array([groups[k].size for k in keys])
    ref_counts = np.array([int(ref[f"count_{k}"]) for k in keys])
    assert chi2_p(counts, ref_counts) > 1e-4, dict(zip(keys, zip(counts, ref_counts)))
    tested = 0
    for k in keys:
        u = groups[k]
        if f"edges_{k}" not in ref.files or u.size < 100:
            continue
        h = np.histogram(u, ref[f"edges_{k}"])[0]
        assert chi2_p(h, ref[f"hist_{k}"]) > 1e-4, (k, h, ref[f"hist_{k}"])
        p = stats.ks_2samp(u, ref[f"sample_{k}"]).pvalue
        assert p > 1e-4, (k, p)
        tested += 1
    assert tested >= 5
