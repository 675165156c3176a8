"""Device event pass (mx_event_coords) against the reference's marx2fits
output and the CPU oracle.

Tolerances: CHIPX/CHIPY, TDETX/TDETY, EXPNO, FLTGRADE and GRADE exact;
DETX/DETY bit-identical to the oracle when the detector does not rotate
(pure arithmetic, no multiply-add contraction on either side), else within
1e-9 pixel.  Sky X/Y within 1e-9 pixel plus the reference formula's own
sensitivity: marx_mnc_to_ra_dec takes the sky angles as acos of values near
1 (pixlib.c:511-521), so one ulp in its argument moves the angle by
ulp / sin(angle); with sin, cos, acos, asin and atan of the device and the
host differing by an ulp, an event a pixel from the aim point may move by
up to 1e-4 pixel.  The single-precision values marx2fits writes are equal
wherever that sensitivity does not reach a rounding boundary.
"""
import os

import numpy as np
import pytest

from oracle.event_coords import PIXADJ, event_coords as oracle_coords, subpix_tables
from marx_gb300.caldb.pack import DEFAULT_PACK, read_pack
from marx_gb300 import workloads as W
from marx_gb300 import events as E

from test_events import CASES, MODES, load_case

pytestmark = pytest.mark.gpu
PIX_TOL = 1e-9
DETECTOR_WORKLOAD = {"ACIS-I": "plain_scatter", "ACIS-S": "plain_hetg", "HRC-I": "plain_hrci", "HRC-S": "letg_hrcs"}


@pytest.fixture(scope="module")
def subpix():
    return subpix_tables(read_pack(DEFAULT_PACK))


_engines = {}


def engine_for(det):
    from marx_gb300._native import Engine
    if det not in _engines:
        _engines[det] = Engine(W.ALL[DETECTOR_WORKLOAD[det]]().cfg)
    return _engines[det]


def run_case(name, mode, subpix):
    z, det, params, ev = load_case(name)
    eng = engine_for(det)
    p = E.params(focal_length=params["focal_length"], det_offset=params["det_offset"], roll_nom=params["roll_nom"],
                 frame_time=params["frame_time"], dithered=params["dithered"], pixel_adjust=mode)
    g = E.event_coords_host(eng, p, dict(ev, uniforms=z["uniforms"]))
    params["pixel_adjust"] = PIXADJ[mode]
    o = oracle_coords(det, z["geom"], z["tdet"], z["fp"], params, ev, z["uniforms"], subpix)
    return z, g, o, ev


def check_against_oracle(g, o, ev, where):
    for c in ("chipx", "chipy", "tdetx", "tdety", "expno", "fltgrade", "grade"):
        np.testing.assert_array_equal(g[c], o[c].astype(g[c].dtype), err_msg=f"{where} {c}")
    still = not np.any(ev["det_theta"])
    for c in ("detx", "dety"):
        if still:
            np.testing.assert_array_equal(g[c], o[c], err_msg=f"{where} {c}")
        else:
            assert np.max(np.abs(g[c] - o[c])) <= PIX_TOL, (where, c)
    tol = sky_tolerance(o)
    for c in ("x", "y"):
        d = np.abs(g[c] - o[c])
        assert np.all(d <= tol[c]), (where, c, float(np.max(d / tol[c])))


FP_DELTA = {4096.5: 0.492, 16384.5: 0.13175, 32768.5: 0.1318}   # arcsec per pixel by fp_x0 (detpix.c:42-63)
ARG_EPS = 1e-15        # a few ulps of the acos arguments, which sit near 1


def sky_tolerance(o, x0=None):
    """1e-9 pixel plus the sensitivity of X (Y) to an ulp-level change of
    the acos argument that gives the sky RA (Dec) offset."""
    x0 = x0 if x0 is not None else min(FP_DELTA, key=lambda c: abs(c - np.median(o["x"])))
    delta = FP_DELTA[x0] * np.pi / 648000.0
    out = {}
    for c in ("x", "y"):
        ang = np.abs(o[c] - x0) * delta
        with np.errstate(divide="ignore"):
            sens = np.minimum(ARG_EPS / np.sin(ang), np.sqrt(2 * ARG_EPS))   # acos(1 - eps) at the pole
        out[c] = PIX_TOL + sens / delta
    return out


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("name", CASES)
def test_events_match_marx2fits(cuda, name, mode, subpix):
    z, g, o, ev = run_case(name, mode, subpix)
    check_against_oracle(g, o, ev, f"{name} {mode}")
    for c in ("chipx", "chipy", "tdetx", "tdety", "detx", "dety", "x", "y", "expno", "fltgrade", "grade"):
        key = f"{mode}_{c}"
        if key not in z:
            continue
        ref = z[key]
        mine = g[c].astype(np.int16) if c in ("chipx", "chipy") else g[c]
        if ref.dtype.kind == "f":
            same = mine.astype(np.float32) == ref
            if c in ("x", "y"):
                # a differing float is one whose sensitivity reaches the rounding boundary
                ulp = np.spacing(np.abs(ref)).astype(np.float64)
                near = np.abs(mine - ref.astype(np.float64)) <= 0.5 * ulp + sky_tolerance(o)[c]
                assert np.all(same | near), (name, mode, c)
                assert same.mean() > 0.995, (name, mode, c, same.mean())
            else:
                np.testing.assert_array_equal(mine.astype(np.float32), ref, err_msg=f"{name} {mode} {c}")
        else:
            np.testing.assert_array_equal(mine.astype(np.int64), ref.astype(np.int64), err_msg=f"{name} {mode} {c}")


@pytest.mark.parametrize("mode", MODES)
def test_hrc_i_events_match_oracle(cuda, mode, subpix):
    z, g, o, ev = run_case("hrc_i", mode, subpix)
    check_against_oracle(g, o, ev, f"hrc_i {mode}")


def synthetic_events(n, geom, seed, frame_time, events_per_frame):
    rng = np.random.default_rng(seed)
    ids = geom[:, 0].astype(np.int64)
    f = np.float32
    t = np.sort(rng.uniform(0, n / events_per_frame * frame_time, n)).astype(f)
    arc = np.pi / 648000.0
    return dict(ccd=ids[rng.integers(0, len(ids), n)].astype(np.int8),
                xpixel=rng.uniform(0, 1024, n).astype(f), ypixel=rng.uniform(0, 1024, n).astype(f), time=t,
                sky_ra=(8 * arc * np.sin(t / 159.0)).astype(f), sky_dec=(8 * arc * np.sin(t / 112.5)).astype(f),
                sky_roll=np.full(n, 1.2, f), det_dy=np.zeros(n, f), det_dz=np.zeros(n, f),
                det_theta=np.zeros(n, f), b_energy=rng.uniform(0.3, 10, n).astype(f)), rng.random((3, n))


@pytest.mark.parametrize("mode", ["EDSER", "EXACT"])
def test_frames_across_blocks(cuda, mode, subpix):
    """Three million ACIS events, frames of ~400 events that straddle the
    pass's 256-event tiles: frame numbers and frame dither like the oracle."""
    z, det, params, _ = load_case("acis_i")
    ev, U = synthetic_events(3_000_000, z["geom"], 7, params["frame_time"], 400)
    eng = engine_for(det)
    p = E.params(focal_length=params["focal_length"], det_offset=params["det_offset"], roll_nom=params["roll_nom"],
                 frame_time=params["frame_time"], dithered=True, pixel_adjust=mode)
    g = E.event_coords_host(eng, p, dict(ev, uniforms=U))
    params["pixel_adjust"] = PIXADJ[mode]
    o = oracle_coords(det, z["geom"], z["tdet"], z["fp"], params, ev, U, subpix)
    check_against_oracle(g, o, ev, f"frames {mode}")


def test_device_entry_on_traced_photons(cuda, subpix):
    """Trace photons, compact the survivors on the device and run the event
    pass on the photon columns through the index: equal to the oracle on the
    host copy of the same columns."""
    import torch
    from marx_gb300._native import DevicePhotons
    z, det, params, _ = load_case("acis_i")
    w = W.ALL["plain_scatter"]()
    eng = engine_for(det)
    n = 200_000
    d = DevicePhotons.from_host(w.photons(n, seed=3))
    eng.trace(d, seed=11)
    idx = eng.compact(d.flags)
    m = idx.numel()
    assert m > 1000
    p = E.params(focal_length=params["focal_length"], det_offset=params["det_offset"], roll_nom=params["roll_nom"],
                 frame_time=params["frame_time"], dithered=True, pixel_adjust="RANDOMIZE", time_offset=12.5)
    U = torch.rand((3, m), dtype=torch.float64, device="cuda")
    g = E.event_coords(eng, p, dict(E.photon_events(d, idx), uniforms=U), m)
    torch.cuda.synchronize()
    g = {k: v.cpu().numpy() for k, v in g.items()}
    q = d.to_host()
    ii = idx.cpu().numpy()
    ev = dict(ccd=q.ccd_num[ii], xpixel=q.y_pixel[ii], ypixel=q.z_pixel[ii],
              time=(q.arrival_time[ii] + 12.5).astype(np.float32), sky_ra=q.dither_state[0][ii],
              sky_dec=q.dither_state[1][ii], sky_roll=q.dither_state[2][ii], det_dy=np.zeros(m, np.float32),
              det_dz=np.zeros(m, np.float32), det_theta=np.zeros(m, np.float32), b_energy=np.zeros(m, np.float32))
    params["pixel_adjust"] = PIXADJ["RANDOMIZE"]
    o = oracle_coords(det, z["geom"], z["tdet"], z["fp"], params, ev, U.cpu().numpy(), subpix)
    check_against_oracle(g, o, ev, "traced photons")


def test_bad_chip_and_empty_list(cuda):
    z, det, params, ev = load_case("acis_i")
    eng = engine_for(det)
    p = E.params(dithered=True, pixel_adjust="EXACT")
    E.bad_count(eng, reset=True)
    assert all(len(v) == 0 for v in E.event_coords_host(eng, p, {k: v[:0] for k, v in ev.items()}, n=0).values())
    bad = {k: v[:10].copy() for k, v in ev.items()}
    bad["ccd"][3] = 7                                   # an ACIS-S chip on an ACIS-I run
    with pytest.raises(RuntimeError):
        E.event_coords_host(eng, p, bad)
    assert E.bad_count(eng) == 1


def test_philox_uniforms_pick_grades_evenly(cuda):
    """Without pre-drawn uniforms the grade draw comes from Philox: corner
    sub-pixels take each of their four flight grades a quarter of the time."""
    z, det, params, _ = load_case("acis_i")
    n = 400_000
    rng = np.random.default_rng(5)
    f = np.float32
    ev = dict(ccd=np.zeros(n, np.int8), xpixel=np.full(n, 100.1, f), ypixel=np.full(n, 200.1, f),
              time=np.sort(rng.uniform(0, 1e4, n)).astype(f))
    g = E.event_coords_host(engine_for(det), E.params(dithered=False, pixel_adjust="EXACT"), ev, seed=99)
    vals, counts = np.unique(g["fltgrade"], return_counts=True)
    assert list(vals) == [10, 11, 138, 139]
    assert np.all(np.abs(counts / n - 0.25) < 0.005)
