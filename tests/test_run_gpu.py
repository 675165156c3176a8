"""mx_run_marx: marx's main loop on the GPU (marx/src/marx.c:545-608).

A parameter file written by the test drives the run.  Checked: the photon
counts and batches NumRays and dNumRays ask for; every written photon equal
to the same source photons traced directly through the engine; identical
output for the same RandomSeed; the ExposureTime stop; the ray file of
DumpToRayFile; and the marx.par and obs.par that marx2fits reads."""
import ctypes as C
import os

import numpy as np
import pytest

from marx_gb300 import config as cfgmod
from marx_gb300.output import read_dir, read_rayfile
from marx_gb300.run import write_par, run_marx

pytestmark = pytest.mark.gpu


def _cfg(dither="INTERNAL"):
    c = cfgmod.default_config()
    c.grating = cfgmod.GRATING["NONE"]
    c.detector = cfgmod.DETECTOR["ACIS-I"]
    c.dither = cfgmod.DITHER[dither]
    c.dither_amp[:] = [8.0, 8.0, 0.0]
    c.dither_period[:] = [1000.0, 707.0, 1e5]
    return c


SRC = dict(SourceRA=250.2134679741175 + 0.5 / 60.0, SourceDEC=-53.75743813458669 - 0.3 / 60.0, MinEnergy=0.3,
           MaxEnergy=8.0, SourceFlux=0.01)


def test_run_counts_batches_and_columns(cuda, tmp_path):
    par = str(tmp_path / "sim.par")
    out = str(tmp_path / "out")
    write_par(par, _cfg(), NumRays=200_000, dNumRays=60_000, OutputDir=out, RandomSeed=11, **SRC)
    st = run_marx(par)
    # whole batches of dNumRays until NumRays are collected (marx.c:564-575)
    assert st["collected"] == 240_000 and st["iterations"] == 4
    d = read_dir(out)
    assert 0.05 * 240_000 < st["detected"] < 0.6 * 240_000
    for k in ("energy", "time", "xpos", "ypos", "zpos", "xcos", "detector", "xpixel", "ypixel", "mirror", "sky_ra",
              "b_energy", "pha"):
        assert d[k].size == st["detected"], k
    assert np.all((d["energy"] >= 0.3) & (d["energy"] <= 8.0))
    assert np.all(np.diff(d["time"].astype(np.float64)) >= 0.0)          # batches follow one another
    assert np.all((d["detector"] >= 0) & (d["detector"] <= 3))            # ACIS-I chips
    assert abs(float(d["time"][-1]) - st["total_time"]) <= 1e-3 * st["total_time"]
    assert st["total_time"] > 0


def test_run_photons_equal_the_direct_trace(cuda, tmp_path):
    """Every photon the run writes is the photon of that tag generated by
    mx_generate_source and traced by mx_trace with the run's seed (no
    dither and no frame-transfer streak, so arrival times do not enter)."""
    import torch
    from marx_gb300._native import Engine, DevicePhotons, load_library
    from marx_gb300.batched import make_source, generate_source
    cfg = _cfg("NONE")
    cfg.acis_frame_transfer_time = 0.0
    par = str(tmp_path / "sim.par")
    out = str(tmp_path / "out")
    n = 30_000
    write_par(par, cfg, NumRays=n, dNumRays=10_000, OutputDir=out, RandomSeed=5, **SRC)
    st = run_marx(par)
    d = read_dir(out)
    L = load_library()
    L.mx_source_direction.argtypes = [C.POINTER(cfgmod.MxConfig), C.c_double, C.c_double, C.POINTER(C.c_double)]
    p = (C.c_double * 3)()
    assert L.mx_source_direction(C.byref(cfg), SRC["SourceRA"], SRC["SourceDEC"], p) == 0
    eng = Engine(cfg)
    src = make_source(p[:], energy=(SRC["MinEnergy"], SRC["MaxEnergy"]))
    dev = DevicePhotons(n)
    generate_source(eng, src, 0, 5, dev)
    eng.trace(dev, stages=15, seed=5)
    torch.cuda.synchronize()
    q = dev.to_host()
    good = (q.flags & 0xFF) == 0
    assert st["detected"] == int(good.sum())
    assert np.array_equal(d["energy"], q.energy[good].astype(np.float32))
    for k, col in (("xpos", q.x[0]), ("ypos", q.x[1]), ("zpos", q.x[2]), ("xcos", q.p[0]), ("ycos", q.p[1])):
        assert np.array_equal(d[k], col[good].astype(np.float32)), k
    assert np.array_equal(d["detector"], q.ccd_num[good])
    assert np.array_equal(d["xpixel"], q.y_pixel[good]) and np.array_equal(d["ypixel"], q.z_pixel[good])


def test_run_is_reproducible_and_seeded(cuda, tmp_path):
    par = str(tmp_path / "sim.par")
    runs = []
    for k, seed in enumerate((3, 3, 4)):
        out = str(tmp_path / f"o{k}")
        write_par(par, _cfg(), NumRays=20_000, dNumRays=20_000, OutputDir=out, RandomSeed=seed, **SRC)
        run_marx(par)
        runs.append({f: open(os.path.join(out, f), "rb").read() for f in sorted(os.listdir(out)) if f.endswith(".dat")})
    assert runs[0] == runs[1]
    assert runs[0]["energy.dat"] != runs[2]["energy.dat"]


def test_run_stops_at_the_exposure_time(cuda, tmp_path):
    par = str(tmp_path / "sim.par")
    out = str(tmp_path / "out")
    write_par(par, _cfg(), NumRays=0, dNumRays=50_000, ExposureTime=2000.0, OutputDir=out, RandomSeed=2, **SRC)
    st = run_marx(par)
    # marx_create_photons keeps the first photon at or past the time left
    assert st["total_time"] >= 2000.0
    # Poisson times at SourceFlux x the mirror's open area (compute_mean_time)
    from marx_gb300.run import geometric_area
    expect = SRC["SourceFlux"] * geometric_area(_cfg()) * st["total_time"]
    assert abs(st["collected"] - expect) < 5 * np.sqrt(expect)
    assert st["iterations"] >= 1


def test_run_writes_marx_par_and_obs_par(cuda, tmp_path):
    par = str(tmp_path / "sim.par")
    out = str(tmp_path / "out")
    write_par(par, _cfg(), NumRays=5000, dNumRays=5000, OutputDir="ignored", RandomSeed=1, **SRC)
    st = run_marx(par, [f"OutputDir={out}", "DetOffsetZ=0.25"])
    mp = {ln.split(",")[0]: ln.split(",")[3] for ln in open(os.path.join(out, "marx.par")).read().splitlines()
          if ln.count(",") >= 3 and not ln.startswith("#")}
    assert mp["OutputDir"] == f'"{out}"' and float(mp["DetOffsetZ"]) == 0.25
    obs = {ln.split(",")[0]: ln for ln in open(os.path.join(out, "obs.par")).read().splitlines() if "," in ln}
    assert '"ACIS-I"' in obs["detnam"] and '"GRADED"' in obs["datamode"]
    tstop = float(obs["tstop"].split(",")[3])
    assert tstop == pytest.approx(st["total_time"], rel=1e-12)
    assert float(obs["sim_z"].split(",")[3]) == 0.25


def test_run_dumps_dithered_rays(cuda, tmp_path):
    par = str(tmp_path / "sim.par")
    rays = str(tmp_path / "sim.rays")
    write_par(par, _cfg(), NumRays=12_000, dNumRays=5000, OutputDir=str(tmp_path / "out"), RandomSeed=9,
              DumpToRayFile=True, RayFile=rays, **SRC)
    st = run_marx(par)
    hist, lists = read_rayfile(rays)
    n = sum(q.n for q in lists)
    assert n == st["collected"] == 15_000          # three whole batches of 5000
    q = lists[0]
    assert np.all(q.dither_state[0] != 0) and np.all(q.flags == 0)
    assert np.all(np.diff(np.concatenate([x.arrival_time for x in lists])) >= 0)   # times across the batches


def test_run_rejects_bad_parameters(cuda, tmp_path):
    par = str(tmp_path / "sim.par")
    write_par(par, _cfg(), NumRays=10, dNumRays=10, OutputDir=str(tmp_path / "o"), **SRC)
    for ov, msg in ((["SourceType=SIMPUT"], "not supported"), (["OutputVectors=EQ"], "not understood"),
                    (["dNumRays=0"], "dNumRays"), (["SpectrumType=PLASMA"], "SpectrumType")):
        with pytest.raises(RuntimeError, match=msg):
            run_marx(par, ov)
