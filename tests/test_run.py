"""A run written by mx_run_marx, read by the reference's own marx2fits.

tests/golden/run_acis_i/ holds the output directory of a small GPU run
(tests/golden/make_run_fixture.py: 20000 photons of a POINT source, FLAT
0.3-8 keV, INTERNAL dither, ACIS-I): the column files, marx.par and
obs.par.  marx2fits (oracle/Makefile target m2f: the reference's program
compiled from its sources, its uniform draws served from a file) turns it
into an event list unchanged; the event columns follow the run's own."""
import os
import subprocess

import numpy as np
import pytest

from marx_gb300.output import read_dir

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RUN = os.path.join(ROOT, "tests", "golden", "run_acis_i")


def test_engine_run_directory_has_every_file():
    d = read_dir(RUN)
    n = d["energy"].size
    assert n > 1000
    for k in ("time", "xpos", "ypos", "zpos", "xcos", "ycos", "zcos", "detector", "xpixel", "ypixel", "sky_ra",
              "sky_dec", "sky_roll", "pha", "b_energy", "mirror"):
        assert d[k].size == n, k
    assert os.path.exists(os.path.join(RUN, "marx.par")) and os.path.exists(os.path.join(RUN, "obs.par"))
    assert np.all(np.diff(d["time"].astype(np.float64)) >= 0)


def test_reference_marx2fits_reads_an_engine_run(tmp_path):
    from oracle.bindings import REF_ROOT, reference_available
    from marx_gb300.caldb.pack import read_fits_bintables
    if not reference_available():
        pytest.skip("the reference checkout is not on this machine")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "m2f", f"REF={REF_ROOT}"], check=True)
    d = read_dir(RUN)
    n = d["energy"].size
    ufile = tmp_path / "u.bin"
    np.random.default_rng(3).random(n).tofile(ufile)     # one flight-grade draw per ACIS event
    out = tmp_path / "evt.fits"
    env = dict(os.environ, MARX_DATA_DIR=os.path.join(REF_ROOT, "marx", "data"), MXREF_UNIFORMS=str(ufile))
    r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "marx2fits"), "--pixadj=NONE", RUN, str(out)], env=env,
                       capture_output=True, text=True)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-2000:])
    ev = next(c for h, c in read_fits_bintables(str(out)) if h.get("EXTNAME") == "EVENTS")
    assert len(ev["TIME"]) == n
    assert np.array_equal(np.asarray(ev["CCD_ID"]).astype(int), d["detector"].astype(int))
    # ACIS events carry the start of their frame: TIMEDEL = ACIS_Exposure_Time
    # + ACIS_Frame_Transfer_Time of the run's marx.par (marx2fits.c:2539-2542,
    # 3438-3439, 3755)
    frame = 3.2 + 0.041
    t = np.asarray(ev["TIME"], dtype=np.float64)
    assert np.allclose(t, frame * np.floor(d["time"].astype(np.float64) / frame), rtol=0, atol=1e-6)
    assert np.all((np.asarray(ev["CHIPX"]) >= 1) & (np.asarray(ev["CHIPX"]) <= 1024))
