"""MARX output directories: the engine's writer (mx_write_photons) against
the files the reference's own writer (marx_write_photons) made for the same
photons, byte for byte (tests/golden/dat_*.npz), and the reader."""
import os

import numpy as np
import pytest

from marx_gb300 import output as O

from helpers import GOLDEN, load_trace_fixture


def traced(name):
    w, ph, U, N, z = load_trace_fixture(name)
    q = ph.copy()
    for k in z.files:
        if hasattr(q, k) and k != "energy":
            getattr(q, k)[...] = z[k]
    return w, q


@pytest.mark.parametrize("name", ["plain_scatter", "letg_hrcs"])
def test_writer_matches_reference_files(tmp_path, name):
    ref = np.load(os.path.join(GOLDEN, f"dat_{name}.npz"))
    w, q = traced(name)
    h = O.history(w.cfg)
    assert h == int(ref["history"])
    O.write_photons(q, h, O.ALL, str(tmp_path), total_time=12.5)
    O.write_photons(q, h, O.ALL, str(tmp_path), append=True, total_time=100.0)
    want = {f for f in ref.files if f.endswith(".dat")}
    assert set(os.listdir(tmp_path)) == want
    for f in want:
        got = np.frombuffer(open(tmp_path / f, "rb").read(), dtype=np.uint8)
        assert np.array_equal(got, ref[f]), f


def test_reader_round_trip(tmp_path):
    w, q = traced("letg_hrcs")
    O.write_photons(q, O.history(w.cfg), O.ALL, str(tmp_path), total_time=5.0)
    cols = O.read_dir(str(tmp_path))
    good = (q.flags & 0xFF) == 0
    assert np.array_equal(cols["xpos"], q.x[0][good].astype(np.float32))
    assert np.array_equal(cols["order"], q.order[good])
    assert np.array_equal(cols["ofine"], q.support_orders[0][good])
    assert np.array_equal(cols["pha"], q.pulse_height[good])
    assert np.array_equal(cols["hrc_u"], q.u_pixel[good])
    assert np.array_equal(cols["time"], (q.arrival_time[good] + 5.0).astype(np.float32))
    assert O.read_column(str(tmp_path / "detector.dat"))[0] == "CCDID"


def test_write_mask_and_empty_list(tmp_path):
    w, q = traced("plain_scatter")
    q.flags[:] = 0x08                          # every photon missed the detector: no rows
    O.write_photons(q, O.history(w.cfg), O.OUT["X"] | O.OUT["ENERGY"], str(tmp_path), dither=False)
    assert sorted(os.listdir(tmp_path)) == ["energy.dat", "xpos.dat", "ypos.dat", "zpos.dat"]
    assert len(O.read_column(str(tmp_path / "xpos.dat"))[1]) == 0


def test_image_fits_reader(tmp_path):
    """The IMAGE source's FITS reader: pixels and scale as the reference's
    open_image_fits_file reads them (CDELT, else the CD matrix, else none)."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_golden import source_image, write_image_fits
    from marx_gb300.batched import read_image_fits
    im, scale = source_image()
    f = tmp_path / "im.fits"
    write_image_fits(str(f), im, scale)
    got, sc = read_image_fits(str(f))
    assert got.dtype == np.float32 and got.shape == im.shape and np.array_equal(got, im)
    assert sc == (abs(-scale[0]), scale[1])
