"""marx2fits's event coordinates on the CPU: the oracle restatement against
the reference's own marx2fits output (tests/golden/events_*.npz), the
ctypes mirror of the C structs, and the fixture's draw-order bookkeeping."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle.event_coords import PIXADJ, event_coords, subpix_tables
from marx_gb300.caldb.pack import DEFAULT_PACK, read_pack

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
CASES = ("acis_i", "acis_s", "acis_i_nodither", "hrc_s")
MODES = ("EXACT", "NONE", "RANDOMIZE", "EDSER")
EVENT_INPUTS = ("ccd", "xpixel", "ypixel", "time", "sky_ra", "sky_dec", "sky_roll", "det_dy", "det_dz",
                "det_theta", "b_energy")


def load_case(name):
    z = np.load(os.path.join(GOLDEN, f"events_{name}.npz"))
    P = z["params"]
    params = dict(focal_length=P[0], det_offset=P[1:4], roll_nom=P[4], frame_time=P[5], dithered=bool(P[6]))
    ev = {k: z[k] for k in EVENT_INPUTS}
    return z, str(z["detector"]), params, ev


@pytest.fixture(scope="module")
def subpix():
    return subpix_tables(read_pack(DEFAULT_PACK))


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_marx2fits(name, mode, subpix):
    """Every column marx2fits wrote (single precision) equals the oracle's."""
    z, det, params, ev = load_case(name)
    params["pixel_adjust"] = PIXADJ[mode]
    o = event_coords(det, z["geom"], z["tdet"], z["fp"], params, ev, z["uniforms"], subpix)
    cols = [c for c in ("chipx", "chipy", "tdetx", "tdety", "detx", "dety", "x", "y", "expno", "fltgrade", "grade")
            if f"{mode}_{c}" in z]
    assert {"chipx", "detx", "x", "tdetx"} <= set(cols)
    for c in cols:
        ref = z[f"{mode}_{c}"]
        mine = o[c]
        if c in ("chipx", "chipy"):          # CHIPX is written as a short (write_float32_as_int16)
            mine = mine.astype(np.int16)
        if ref.dtype.kind == "f":
            np.testing.assert_array_equal(mine.astype(np.float32), ref, err_msg=f"{name} {mode} {c}")
        else:
            np.testing.assert_array_equal(mine.astype(np.int64), ref.astype(np.int64), err_msg=f"{name} {mode} {c}")


def test_frames_share_the_first_events_dither():
    """ACIS with a pixel adjustment other than EXACT: an event's dither is
    that of its frame's first event (read_dither_value), so shuffling the
    dither inside a frame leaves the first event's coordinates only."""
    z, det, params, ev = load_case("acis_i")
    params["pixel_adjust"] = PIXADJ["NONE"]
    U = z["uniforms"]
    sub = subpix_tables(read_pack(DEFAULT_PACK))
    a = event_coords(det, z["geom"], z["tdet"], z["fp"], params, ev, U, sub)
    expno = a["expno"]
    first = np.r_[True, expno[1:] != expno[:-1]]
    assert 50 < first.sum() < len(expno) // 5          # frames of several events
    ev2 = dict(ev)
    for c in ("sky_ra", "sky_dec", "sky_roll"):
        v = ev[c].copy()
        v[~first] = v[~first] * np.float32(3.0) + np.float32(1e-5)
        ev2[c] = v
    b = event_coords(det, z["geom"], z["tdet"], z["fp"], params, ev2, U, sub)
    np.testing.assert_array_equal(a["x"], b["x"])
    params["pixel_adjust"] = PIXADJ["EXACT"]
    c1 = event_coords(det, z["geom"], z["tdet"], z["fp"], params, ev, U, sub)
    c2 = event_coords(det, z["geom"], z["tdet"], z["fp"], params, ev2, U, sub)
    assert np.all(c1["x"][~first] != c2["x"][~first])


def test_hrc_i_fixture_records_the_reference_failure():
    """The reference's marx2fits cannot open an HRC-I run (its detector
    set-up reads a parameter from a null file); the fixture keeps inputs and
    geometry for the oracle-only comparison."""
    z = np.load(os.path.join(GOLDEN, "events_hrc_i.npz"))
    assert "fails" in str(z["marx2fits"])
    assert z["geom"].shape[0] == 1 and not any(k.startswith("EXACT_") for k in z.files)


def test_event_structs_match_the_header(tmp_path):
    """ctypes layouts of mx_event_params and mx_events equal the C compiler's."""
    from marx_gb300.events import EventParams, MxEvents
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = [f for f, _ in MxEvents._fields_]
    pfields = [f for f, _ in EventParams._fields_]
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "marx_gb300.h"', 'int main(void) {',
           'printf("%zu %zu\\n", sizeof(mx_events), sizeof(mx_event_params));']
    src += [f'printf("%zu\\n", offsetof(mx_events, {f}));' for f in fields]
    src += [f'printf("%zu\\n", offsetof(mx_event_params, {f}));' for f in pfields]
    src += ["return 0; }"]
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    import ctypes as C
    assert int(out[0]) == C.sizeof(MxEvents) and int(out[1]) == C.sizeof(EventParams)
    offs = [int(v) for v in out[2:]]
    assert offs[:len(fields)] == [getattr(MxEvents, f).offset for f in fields]
    assert offs[len(fields):] == [getattr(EventParams, f).offset for f in pfields]


def test_subpix_tables_in_the_pack():
    S = read_pack(DEFAULT_PACK)
    t = subpix_tables(S)
    assert set(t) == {"fi", "bi"}
    assert 0 in t["fi"] and 10 in t["bi"]
    for d in t.values():
        for e, dx, dy in d.values():
            assert len(e) >= 2 and np.all(np.diff(e) > 0)


def test_marx2fits_reads_the_engines_output_directory(tmp_path):
    """The traced photons of a parity fixture (which the device trace
    reproduces bit for bit), written by mx_write_photons with the run's
    marx.par and obs.par (write_run_files): the reference's own marx2fits
    reads the directory unchanged, and its event columns equal the oracle's
    on the columns read back."""
    from oracle import bindings
    if not bindings.reference_available():
        pytest.skip("needs the reference's sources to build marx2fits")
    bindings.build_reference()
    from helpers import load_trace_fixture
    from marx_gb300 import output as O
    from marx_gb300.caldb.pack import read_fits_bintables
    w, ph, U, N, z = load_trace_fixture("plain_scatter")
    q = ph.copy()
    for k in z.files:
        if hasattr(q, k) and k != "energy":
            getattr(q, k)[...] = z[k]
    d = str(tmp_path / "sim")
    O.write_photons(q, O.history(w.cfg), O.ALL, d, total_time=0.0)
    ref_root = bindings.REF_ROOT
    O.write_run_files(d, w.cfg, os.path.join(ref_root, "marx", "par", "marx.par"),
                      os.path.join(ref_root, "marx", "data"), 1000.0)
    cols = O.read_dir(d)
    n = len(cols["time"])
    assert n > 100
    u = np.random.default_rng(2).random((3, n))
    ufile = tmp_path / "u.bin"
    u[0].astype(np.float64).tofile(ufile)              # one grade draw per ACIS event (EXACT)
    out = tmp_path / "evt.fits"
    env = dict(os.environ, MARX_DATA_DIR=os.path.join(ref_root, "marx", "data"), MXREF_UNIFORMS=str(ufile))
    r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "marx2fits"), "--pixadj=EXACT", d, str(out)],
                       env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    ev_fits = next(c for h, c in read_fits_bintables(str(out)) if h.get("EXTNAME") == "EVENTS")
    zc, det, _, _ = load_case("acis_i")
    zero = np.zeros(n, np.float32)
    ev = dict(ccd=cols["detector"], xpixel=cols["xpixel"], ypixel=cols["ypixel"], time=cols["time"],
              sky_ra=cols["sky_ra"], sky_dec=cols["sky_dec"], sky_roll=cols["sky_roll"], det_dy=zero, det_dz=zero,
              det_theta=zero, b_energy=zero)
    params = dict(focal_length=10070.0, det_offset=tuple(w.cfg.det_offset), roll_nom=w.cfg.roll_nom,
                  frame_time=3.2 + 0.041, dithered=True, pixel_adjust=PIXADJ["EXACT"])
    o = event_coords("ACIS-I", zc["geom"], zc["tdet"], zc["fp"], params, ev, u)
    for c in ("DETX", "DETY", "X", "Y"):
        np.testing.assert_array_equal(o[c.lower()].astype(np.float32), ev_fits[c], err_msg=c)
    for c in ("CHIPX", "CHIPY"):
        np.testing.assert_array_equal(o[c.lower()].astype(np.int16), ev_fits[c], err_msg=c)
    for c in ("TDETX", "TDETY", "EXPNO", "FLTGRADE", "GRADE"):
        np.testing.assert_array_equal(o[c.lower()].astype(np.int64), ev_fits[c].astype(np.int64), err_msg=c)
