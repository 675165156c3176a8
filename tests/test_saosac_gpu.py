"""SAOSAC rays on the GPU: the photons the reader makes of the synthetic ray
file traced from the grating on (the rays have passed the mirror) against
the oracle's trace of the same photons and Philox draws, and mx_run_marx
with SourceType SAOSAC writing exactly the photons of that trace."""
import os

import numpy as np
import pytest

from marx_gb300 import workloads as W
from marx_gb300.saosac import SaosacFile

from helpers import assert_parity

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STAGES = 1 | 4 | 8     # dither, grating, detector


def _rays(cfg):
    s = SaosacFile(os.path.join(GOLDEN, "saosac_synthetic.fits"), cfg.hrma_cap_x)
    q = s.read(s.rows, seed=21)
    s.close()
    return q


def _config():
    # every order of the efficiency tables (a parameter file cannot limit
    # them) and no roll: the dither turns the rays' directions about the
    # axis, not their positions on the cap (as _marx_dither_photons does),
    # so a roll would send rays that converge on the focus elsewhere
    w = W.plain_hetg(parity=True)
    w.cfg.roll_nom = 0.0
    return w


def test_saosac_rays_through_grating_and_detector_match_oracle(cuda):
    import torch
    from marx_gb300._native import Engine, DevicePhotons
    from oracle.bindings import Oracle
    w = _config()
    ph = _rays(w.cfg)
    assert ph.n == 2998 and set(np.unique(ph.mirror_shell)) == {0, 1, 2, 3}
    a = ph.copy()
    Oracle(w.cfg).trace(a, stages=STAGES, seed=8)
    d = DevicePhotons.from_host(ph)
    Engine(w.cfg).trace(d, stages=STAGES, seed=8)
    torch.cuda.synchronize()
    q = d.to_host()
    assert_parity(q, a, "saosac rays, grating and detector")
    good = (q.flags & 0xFF) == 0
    assert good.sum() > 100 and len(np.unique(q.order[good])) > 3


def test_run_with_saosac_source(cuda, tmp_path):
    import torch
    from marx_gb300._native import Engine, DevicePhotons
    from marx_gb300.output import read_dir
    from marx_gb300.run import write_par, run_marx
    w = _config()
    par = str(tmp_path / "s.par")
    out = str(tmp_path / "out")
    write_par(par, w.cfg, NumRays=5000, dNumRays=1000, OutputDir=out, RandomSeed=21, SourceType="SAOSAC")
    st = run_marx(par, [f"SAOSACFile={os.path.join(GOLDEN, 'saosac_synthetic.fits')}"])
    assert st["collected"] == 2998 and st["iterations"] == 3
    # the same rays in the same batches, traced directly
    s = SaosacFile(os.path.join(GOLDEN, "saosac_synthetic.fits"), w.cfg.hrma_cap_x)
    eng = Engine(w.cfg)
    good = []
    start = 0.0
    while True:
        ph = s.read(1000, seed=21)
        if ph is None:
            break
        eng.set_start_time(start)
        d = DevicePhotons.from_host(ph)
        eng.trace(d, stages=STAGES, seed=21)
        torch.cuda.synchronize()
        q = d.to_host()
        g = (q.flags & 0xFF) == 0
        good.append((q.x[:, g], q.energy[g], q.ccd_num[g], q.order[g]))
        start += float(ph.arrival_time[-1])
    dd = read_dir(out)
    x = np.concatenate([g[0] for g in good], axis=1)
    assert st["detected"] == x.shape[1] == dd["xpos"].size
    assert np.array_equal(dd["ypos"], x[1].astype(np.float32)) and np.array_equal(dd["zpos"], x[2].astype(np.float32))
    assert np.array_equal(dd["order"], np.concatenate([g[3] for g in good]))
