"""The strut screens at the bar edges.

The strut shadows (hrma.c:928-968) are first tested in single precision and
decided there unless a ray passes within 0.05 mm of a bar edge; the cap
struts' screen also forms the MARX-frame coordinates in single precision.
Random photons rarely come that close, so here the aperture angle's
pre-drawn variate (project_photon_to_hrma, hrma.c:984-1050: vignetting,
shell, radius, then the angle) puts every photon within 0.035 rad of one
of the twelve spokes of the three strut sets.  Thousands of rays then pass
within the margin of an edge of the pre-collimator, cap or post-collimator
bars and take the double-precision test.  The GPU trace, fused and
wavefront, must give the oracle's flags, shells, chips and pixels and its
positions within 1e-9 mm.
"""
import numpy as np
import pytest

from marx_gb300 import workloads as W
from marx_gb300.photons import predraw_variates, PHOTON_MIRROR_VBLOCKED, BAD_PHOTON_MASK

from helpers import assert_parity

pytestmark = pytest.mark.gpu


def _edge_photons(w, n, theta_slot, seed):
    ph = w.photons(n, seed=seed)
    U, N = predraw_variates(n, seed + 1)
    rng = np.random.default_rng(seed + 2)
    # spokes every 30 degrees; the aperture angle is 2 pi (u - 1/8)
    phi = rng.integers(0, 12, n) * (np.pi / 6) + rng.uniform(-0.035, 0.035, n)
    U[theta_slot] = np.mod(phi / (2 * np.pi) + 0.125, 1.0)
    return ph, U, N


@pytest.mark.parametrize("name,theta_slot", [("plain_scatter", 3), ("plain_hetg", 3)])
@pytest.mark.parametrize("mode", [1, 2])
def test_strut_edges_match_oracle(cuda, name, theta_slot, mode):
    import torch
    from marx_gb300._native import DevicePhotons, Engine
    from oracle.bindings import Oracle
    w = W.PLAIN[name]()
    n = 50_000
    ph, U, N = _edge_photons(w, n, theta_slot, seed=21)
    ref = ph.copy()
    Oracle(w.cfg).trace(ref, stages=w.stages, U=U, N=N, seed=4)
    blocked = float(np.mean((ref.flags & PHOTON_MIRROR_VBLOCKED) != 0))
    # the angles were aimed at the bars: far more photons are shadowed than
    # the few per cent of a uniform aperture
    assert blocked > 0.2, blocked
    assert int(((ref.flags & BAD_PHOTON_MASK) == 0).sum()) > n // 50
    eng = Engine(w.cfg)
    eng.set_mode(mode)
    d = DevicePhotons.from_host(ph)
    eng.trace(d, stages=w.stages, U=torch.from_numpy(U).cuda(), N=torch.from_numpy(N).cuda(), seed=4)
    torch.cuda.synchronize()
    assert_parity(d.to_host(), ref, f"{name} strut edges, mode {mode}", pixel_ulps=1)
