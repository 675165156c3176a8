"""Differentiable form on the GPU, through the C ABI (mx_diff_*):

  * the weighted rays against the reference's own mirror stage (golden
    fixture, theta = 0 and perturbed) and against the CPU restatement;
  * the rays against the plain trace (mx_trace) of photons of the same tags;
  * the forward image against the CPU restatement's image;
  * the adjoint against central finite differences of the same (replayed)
    function at the full workload, 4e6 rays, at <= 1e-3 relative error;
  * the torch.autograd.Function of the test harness;
  * repeatability and argument checks."""
import os

import numpy as np
import pytest

from marx_gb300.diff import (DiffImage, diff_mirror_config, diff_workload, fd_gradient, source_direction,
                             NPARAM, RECORD, REPLAY, FRESH, PARAM_NAMES)

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
X_TOL_MM = 1e-9
W_RTOL = 1e-12
GRAD_RTOL = 1e-3   # adjoint vs central finite differences, per parameter


@pytest.fixture(scope="module")
def engines(cuda):
    from marx_gb300._native import Engine
    return {"ideal": Engine(diff_mirror_config(ideal=True)), "reflect": Engine(diff_mirror_config(ideal=False))}


def _rays(eng, cfg, theta, mode=FRESH):
    d = DiffImage(eng, cfg)
    yzw = d.rays(theta, mode).cpu().numpy()
    d.close()
    return yzw


@pytest.mark.parametrize("mirror", ["ideal", "reflect"])
@pytest.mark.parametrize("which", ["zero", "true"])
def test_rays_match_reference(engines, mirror, which):
    g = np.load(os.path.join(HERE, "golden", "diff_rays.npz"))
    w = diff_workload(n_rays=int(g["n"]))
    yzw = _rays(engines[mirror], w.cfg, g[f"{mirror}_{which}_theta"])
    ry, rz = g[f"{mirror}_{which}_y"], g[f"{mirror}_{which}_z"]
    ref_hit = np.isfinite(ry)
    hit = yzw[2] > 0
    if mirror == "ideal":
        assert np.array_equal(hit, ref_hit)
    else:
        assert not np.any(ref_hit & ~hit)
    d = max(np.abs(yzw[0][ref_hit] - ry[ref_hit]).max(), np.abs(yzw[1][ref_hit] - rz[ref_hit]).max())
    assert d <= X_TOL_MM, d


@pytest.mark.parametrize("which", ["zero", "true"])
def test_rays_and_image_match_oracle(engines, which):
    from oracle.bindings import Oracle
    w = diff_workload(n_rays=200_000)
    theta = np.zeros(NPARAM) if which == "zero" else w.theta_true
    eng = engines["reflect"]
    d = DiffImage.centred(eng, w.cfg)
    o = Oracle(diff_mirror_config(ideal=False))
    yzw = d.rays(theta, FRESH).cpu().numpy()
    oy, oimg = o.weighted(d.cfg, theta)
    hit, ohit = yzw[2] > 0, oy[2] > 0
    assert np.array_equal(hit, ohit)
    assert np.abs(yzw[0][hit] - oy[0][hit]).max() <= X_TOL_MM
    assert np.abs(yzw[1][hit] - oy[1][hit]).max() <= X_TOL_MM
    assert np.abs(yzw[2][hit] / oy[2][hit] - 1.0).max() <= W_RTOL
    img = d.forward(theta, FRESH).cpu().numpy()
    # the same fixed-point splat on both sides: equal but for the last bits
    # of a ray's FP64 position or weight moving a tap by one unit
    assert np.abs(img - oimg).max() <= 1e-9 * oimg.max()
    assert img.sum() == pytest.approx(oimg.sum(), rel=1e-12)


def test_rays_match_plain_trace(engines):
    """The weighted ray of tag i is the plain trace's photon of tag i: same
    aperture point, same conics (ideal mirror: nothing absorbed)."""
    import torch
    from marx_gb300._native import DevicePhotons
    from marx_gb300.photons import PhotonList
    eng = engines["ideal"]
    w = diff_workload(n_rays=100_000)
    n = w.cfg.n_rays
    p0 = source_direction(w.cfg.src_y, w.cfg.src_z)
    ph = PhotonList.from_inputs(np.full(n, w.cfg.energy), np.repeat(p0[:, None], n, 1), np.zeros(n))
    ph.tag[:] = np.arange(n, dtype=np.uint32)
    dp = DevicePhotons.from_host(ph)
    eng.trace(dp, stages=2, seed=w.cfg.seed)
    torch.cuda.synchronize()
    q = dp.to_host()
    good = (q.flags & 0xFF) == 0
    t = -q.x[0] / q.p[0]
    yzw = _rays(eng, w.cfg, np.zeros(NPARAM))
    hit = yzw[2] > 0
    assert np.array_equal(hit, good)
    assert np.abs(yzw[0][hit] - (q.x[1] + t * q.p[1])[hit]).max() <= X_TOL_MM
    assert np.abs(yzw[1][hit] - (q.x[2] + t * q.p[2])[hit]).max() <= X_TOL_MM


@pytest.fixture(scope="module")
def c5(engines):
    """The full differentiable workload: 4e6 rays, target image at the
    seeded perturbation from rays of another seed."""
    import torch
    eng = engines["reflect"]
    w = diff_workload()
    d = DiffImage.centred(eng, w.cfg)
    tc = d.cfg.copy()
    tc.seed = w.target_seed
    dt = DiffImage(eng, tc)
    target = dt.forward(w.theta_true, FRESH).clone()
    dt.close()
    torch.cuda.synchronize()
    return w, d, target


def _grad_errors(g_adj, g_fd):
    rel = np.abs(g_adj - g_fd) / np.maximum(np.abs(g_fd), 1e-300)
    norm = np.linalg.norm(g_adj - g_fd) / np.linalg.norm(g_fd)
    return rel, norm


@pytest.mark.parametrize("at", ["zero", "random"])
def test_adjoint_matches_central_differences(c5, at):
    w, d, target = c5
    theta = np.zeros(NPARAM) if at == "zero" else np.random.default_rng(7).normal(0.0, 1.0, NPARAM)
    img = d.forward(theta, RECORD)
    loss, dl = d.mse(img, target)
    g_adj = d.adjoint(theta, dl)
    g_fd = fd_gradient(d, theta, target, h=2e-3, mode=REPLAY)
    rel, norm = _grad_errors(g_adj, g_fd)
    table = "\n".join(f"{PARAM_NAMES[k]:>10s} {g_adj[k]: .6e} {g_fd[k]: .6e} {rel[k]:.2e}" for k in range(NPARAM))
    print(f"\nloss {float(loss):.6e}  norm-wise rel err {norm:.2e}\n{table}")
    assert norm <= GRAD_RTOL
    assert np.all(rel <= GRAD_RTOL), table


def test_boundary_terms_are_small(c5):
    """Central differences with the decisions made afresh at every step
    include rays crossing the conic edges and strut shadows, which the
    adjoint leaves out; at the workload's scale they stay a small part."""
    w, d, target = c5
    theta = np.zeros(NPARAM)
    img = d.forward(theta, RECORD)
    _, dl = d.mse(img, target)
    g_adj = d.adjoint(theta, dl)
    g_free = fd_gradient(d, theta, target, h=2e-2, mode=FRESH)
    _, norm = _grad_errors(g_adj, g_free)
    print(f"\nadjoint vs free central differences: norm-wise rel {norm:.2e}")
    assert norm <= 5e-2


def test_autograd_function(c5):
    import torch
    from diff_harness import WeightedImage
    w, d, target = c5
    theta = torch.tensor(w.theta_true * 0.5, dtype=torch.float64, device="cuda", requires_grad=True)
    img = WeightedImage.apply(theta, d)
    loss = ((img - target) ** 2).mean()
    loss.backward()
    direct_img = d.forward(theta.detach().cpu().numpy(), RECORD)
    dl_loss, dl = d.mse(direct_img, target)
    g = d.adjoint(theta.detach().cpu().numpy(), dl)
    assert float(loss.detach()) == pytest.approx(float(dl_loss), rel=1e-12)
    np.testing.assert_allclose(theta.grad.cpu().numpy(), g, rtol=1e-12, atol=0)


def test_repeatable(c5):
    w, d, target = c5
    a = d.forward(w.theta_true, RECORD).clone()
    b = d.forward(w.theta_true, RECORD).clone()
    assert bool((a == b).all())
    _, dl = d.mse(a, target)
    assert np.array_equal(d.adjoint(w.theta_true, dl), d.adjoint(w.theta_true, dl))
    # replaying the recorded decisions at the same theta gives the same image
    c = d.forward(w.theta_true, REPLAY)
    assert bool((a == c).all())


def test_argument_checks(engines):
    import torch
    from marx_gb300.diff import MxDiffConfig
    w = diff_workload(n_rays=1000)
    eng = engines["reflect"]
    bad = w.cfg.copy()
    bad.sigma = 2.0
    with pytest.raises(RuntimeError, match="sigma"):
        DiffImage(eng, bad)
    bad = w.cfg.copy()
    bad.n_rays = 0
    with pytest.raises(RuntimeError, match="n_rays"):
        DiffImage(eng, bad)
    d = DiffImage(eng, w.cfg)
    img = d.new_image()
    with pytest.raises(RuntimeError, match="RECORD"):
        d.forward(np.zeros(NPARAM), REPLAY, out=img)
    with pytest.raises(RuntimeError, match="RECORD"):
        d.adjoint(np.zeros(NPARAM), torch.zeros_like(img))
    t = np.zeros(NPARAM)
    t[3] = np.nan
    with pytest.raises(RuntimeError, match="theta"):
        d.forward(t, RECORD, out=img)
    assert isinstance(MxDiffConfig(), MxDiffConfig)


def _thetas(w):
    return {"true": w.theta_true, "random": np.random.default_rng(7).normal(0.0, 1.0, NPARAM)}


@pytest.mark.parametrize("at", ["true", "random"])
def test_adjoint_matches_reference_crn_differences(engines, at):
    """The adjoint against central differences of the reference itself
    (tests/golden/diff_fd_reference.npz): 2e5 rays through the reference's
    ideal mirror with each parameter moved by +-2e-3 in the HRMA geometry
    file, the same rays (Philox variates of their tags) at every step, the
    reference's own decisions at every step, imaged with the engine's
    splat and compared with the same target image by MSE."""
    import torch
    z = np.load(os.path.join(HERE, "golden", "diff_fd_reference.npz"))
    w = diff_workload(n_rays=int(z["n"]))
    cfg = w.cfg.copy()
    cfg.center_y, cfg.center_z = (float(v) for v in z["center"])
    d = DiffImage(engines["ideal"], cfg)
    target = torch.from_numpy(z["target"]).cuda()
    theta = z[f"{at}_theta"]
    img = d.forward(theta, RECORD)
    loss, dl = d.mse(img, target)
    assert float(loss) == pytest.approx(float(z[f"{at}_loss"]), rel=1e-9)
    g_adj = d.adjoint(theta, dl)
    g_ref = z[f"{at}_grad"]
    assert int(z[f"{at}_changed"].sum()) == 0      # no ray changed its hit or miss across a step
    rel, norm = _grad_errors(g_adj, g_ref)
    table = "\n".join(f"{PARAM_NAMES[k]:>10s} {g_adj[k]: .6e} {g_ref[k]: .6e} {rel[k]:.2e}" for k in range(NPARAM))
    print(f"\nadjoint vs reference CRN differences, norm-wise rel {norm:.2e}\n{table}")
    assert np.all(rel <= GRAD_RTOL), table
    d.close()


@pytest.mark.parametrize("at", ["true", "random"])
def test_adjoint_matches_oracle_crn_differences(engines, at):
    """The adjoint of the reflecting mirror (reflectivity weights) on 1e6
    rays against central differences of the oracle's weighted images (the
    restatement pinned to the reference's perturbed-geometry rays), the
    same rays at every step and decisions made afresh, as the reference
    makes them, with a step across which no ray's decisions change."""
    from oracle.bindings import Oracle
    w = diff_workload(n_rays=1_000_000)
    d = DiffImage.centred(engines["reflect"], w.cfg)
    tc = d.cfg.copy()
    tc.seed = w.target_seed
    dt = DiffImage(engines["reflect"], tc)
    target = dt.forward(w.theta_true, FRESH).clone()
    dt.close()
    theta = _thetas(w)[at]
    img = d.forward(theta, RECORD)
    _, dl = d.mse(img, target)
    g_adj = d.adjoint(theta, dl)
    o = Oracle(diff_mirror_config(ideal=False))
    T = target.cpu().numpy()
    # a step small enough that no ray changes between hitting and missing a
    # mirror end or strut across it (such a ray adds a jump, the boundary
    # term the adjoint of the smooth function leaves out; at 1e6 rays and
    # a step of 2e-3 a few rays do)
    h = 5e-4
    g_fd = np.zeros(NPARAM)
    for k in range(NPARAM):
        L, hit = [], []
        for s in (-1.0, 1.0):
            t = theta.copy()
            t[k] += s * h
            yzw, im = o.weighted(d.cfg, t)
            L.append(np.mean((im - T) ** 2))
            hit.append(yzw[2] > 0)
        assert np.array_equal(hit[0], hit[1]), (PARAM_NAMES[k], int(np.sum(hit[0] != hit[1])))
        g_fd[k] = (L[1] - L[0]) / (2.0 * h)
    rel, norm = _grad_errors(g_adj, g_fd)
    table = "\n".join(f"{PARAM_NAMES[k]:>10s} {g_adj[k]: .6e} {g_fd[k]: .6e} {rel[k]:.2e}" for k in range(NPARAM))
    print(f"\nadjoint vs oracle CRN differences, norm-wise rel {norm:.2e}\n{table}")
    assert np.all(rel <= GRAD_RTOL), table
    d.close()
