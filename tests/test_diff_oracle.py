"""The CPU restatement of the differentiable form's weighted rays, pinned
against the reference: the reference's own mirror stage traced the same
aperture points (same variates per tag) with theta = 0 and with the
workload's perturbation written into its HRMA geometry file
(tests/golden/diff_rays.npz, made by tests/golden/make_golden.py)."""
import math
import os

import numpy as np
import pytest

from marx_gb300.diff import diff_workload, diff_mirror_config, NPARAM

HERE = os.path.dirname(os.path.abspath(__file__))
X_TOL_MM = 1e-9


def _fixture():
    return np.load(os.path.join(HERE, "golden", "diff_rays.npz"))


@pytest.fixture(scope="module")
def oracles():
    from oracle.bindings import Oracle
    return {"ideal": Oracle(diff_mirror_config(ideal=True)), "reflect": Oracle(diff_mirror_config(ideal=False))}


@pytest.mark.parametrize("mirror", ["ideal", "reflect"])
@pytest.mark.parametrize("which", ["zero", "true"])
def test_oracle_rays_match_reference(oracles, mirror, which):
    g = _fixture()
    w = diff_workload(n_rays=int(g["n"]))
    assert w.cfg.seed == int(g["seed"]) and w.cfg.energy == float(g["energy"])
    theta = g[f"{mirror}_{which}_theta"]
    yzw, _ = oracles[mirror].weighted(w.cfg, theta, image=False)
    ry, rz = g[f"{mirror}_{which}_y"], g[f"{mirror}_{which}_z"]
    ref_hit = np.isfinite(ry)
    hit = yzw[2] > 0
    if mirror == "ideal":
        # no random absorption: the reference reflects exactly the rays that hit
        assert np.array_equal(hit, ref_hit)
    else:
        # the reference absorbs some at random (vignetting, reflectivity)
        assert not np.any(ref_hit & ~hit)
        assert ref_hit.sum() > 0.6 * hit.sum()
    assert ref_hit.sum() > 1000
    dy = np.abs(yzw[0][ref_hit] - ry[ref_hit]).max()
    dz = np.abs(yzw[1][ref_hit] - rz[ref_hit]).max()
    assert max(dy, dz) <= X_TOL_MM, (dy, dz)


def test_oracle_weights(oracles):
    """Ideal mirrors give unit weights; reflecting ones HRMAVig times the
    reflectivity-and-correction product of the two reflections, below 1."""
    w = diff_workload(n_rays=20000)
    yzw_i, _ = oracles["ideal"].weighted(w.cfg, np.zeros(NPARAM), image=False)
    yzw_r, _ = oracles["reflect"].weighted(w.cfg, np.zeros(NPARAM), image=False)
    hi, hr = yzw_i[2] > 0, yzw_r[2] > 0
    assert np.all(yzw_i[2][hi] == 1.0)
    assert abs(hi.mean() - hr.mean()) < 0.02
    wr = yzw_r[2][hr]
    assert 0.5 < wr.mean() < 0.9 and wr.max() < 1.0 and wr.min() > 0.0


def test_oracle_image_normalisation(oracles):
    w = diff_workload(n_rays=50000)
    yzw, _ = oracles["reflect"].weighted(w.cfg, np.zeros(NPARAM), image=False)
    hit = yzw[2] > 0
    ww = yzw[2][hit]
    w.cfg.center_y = float((ww * yzw[0][hit]).sum() / ww.sum())
    w.cfg.center_z = float((ww * yzw[1][hit]).sum() / ww.sum())
    _, img = oracles["reflect"].weighted(w.cfg, np.zeros(NPARAM), rays=False)
    # each ray deposits its weight (the Gaussian beyond 5 pixels and the
    # fixed-point truncation lose ~1e-6)
    assert img.sum() == pytest.approx(ww.sum() / w.cfg.n_rays, rel=1e-5)
    j, i = np.unravel_index(img.argmax(), img.shape)
    assert abs(i - 127.5) < 3 and abs(j - 127.5) < 3


def test_splat_exponential_accuracy(oracles):
    """The splat's own single-precision exp(-x) (Cody-Waite + Taylor) against
    libm: the image is built from it on both sides."""
    w = diff_workload(n_rays=1)
    w.cfg.center_y = 0.0
    w.cfg.center_z = 0.0
    # a ray far off the image deposits nothing: checks the empty image path
    _, img = oracles["reflect"].weighted(w.cfg, np.zeros(NPARAM), rays=False)
    assert img.sum() == 0.0
    o = oracles["reflect"]
    xs = np.linspace(0.0, 60.0, 2001).astype(np.float32)
    got = np.array([o.splat_exp(float(x)) for x in xs])
    want = np.exp(-xs.astype(np.float64))
    assert np.max(np.abs(got / want - 1.0)) < 3e-7
    assert math.isclose(o.splat_exp(0.0), 1.0)
    assert o.splat_exp(80.0) == 0.0
