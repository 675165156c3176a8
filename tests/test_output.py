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


def _traced_list():
    w, ph, U, N, z = load_trace_fixture("plain_scatter")
    q = ph.copy()
    for k in z.files:
        if hasattr(q, k) and k != "energy":
            getattr(q, k)[...] = z[k]
    q.pi[:] = np.linspace(0.1, 7.0, q.n).astype(np.float32)
    return w, q


def test_rayfile_matches_reference_writer(tmp_path):
    """mx_write_rayfile writes the bytes the reference's
    marx_dump_to_rayfile writes (header and 136-byte records), new and
    appended."""
    from oracle import bindings
    if not bindings.reference_available():
        pytest.skip("needs the reference's sources")
    from oracle.bindings import Reference
    w, q = _traced_list()
    h = O.history(w.cfg)
    mine, ref = str(tmp_path / "mine.ray"), str(tmp_path / "ref.ray")
    O.write_rayfile(q, h, mine, total_time=3.5)
    O.write_rayfile(q, h, mine, append=True, total_time=40.0)
    R = Reference(w.cfg)
    R.dump_rayfile(q, h, ref, new=True, total_time=3.5)
    R.dump_rayfile(q, h, ref, new=False, total_time=40.0)
    a, b = open(mine, "rb").read(), open(ref, "rb").read()
    good = int(((q.flags & 0xFF) == 0).sum())
    assert len(a) == 16 + 2 * good * 136 and a == b


def test_rayfile_round_trip_and_reference_source(tmp_path):
    """Read back in batches with the RAYFILE source's arrival times; the
    reference's RAYFILE source reads the engine's file to the same
    energies and directions."""
    w, q = _traced_list()
    path = str(tmp_path / "rays.ray")
    O.write_rayfile(q, 0x1234, path, total_time=2.0)
    good = (q.flags & 0xFF) == 0
    hist, parts = O.read_rayfile(path, batch=70)
    assert hist == 0x1234 and sum(p.n for p in parts) == good.sum()
    r = {k: np.concatenate([getattr(p, k) for p in parts], axis=-1) for k in ("energy", "x", "p", "tag", "pi", "y_pixel")}
    for k in ("energy", "x", "p", "tag", "pi", "y_pixel"):
        assert np.array_equal(r[k], getattr(q, k)[..., good]), k
    # arrival times: relative to the previous batch's last photon
    t = q.arrival_time[good] + 2.0
    start = 0
    last = 0.0
    for p in parts:
        assert np.array_equal(p.arrival_time, t[start:start + p.n] - last)
        last = t[start + p.n - 1]
        start += p.n
    from oracle import bindings
    if not bindings.reference_available():
        return
    from oracle.bindings import Reference
    n = int(good.sum())
    R = Reference(w.cfg, extra_par={"SourceType": "RAYFILE", "RayFile": path, "DumpToRayFile": "no"})
    _, e, pp = R.source_photons(n, np.full((4, n), 0.5))
    assert np.array_equal(e, q.energy[good]) and np.array_equal(pp, q.p[:, good])
