"""The ASPSOL reader (DitherModel = FILE) on the CPU: the synthetic aspect
solution the fixtures were made with, its keywords, and the configuration
the file implies."""
import os

import numpy as np
import pytest

from marx_gb300.aspsol import ASPSOL_COLUMNS, apply_to_config, read_aspsol
from marx_gb300.config import DITHER, default_config

from helpers import GOLDEN

ASPSOL_FILE = os.path.join(GOLDEN, "aspsol_synthetic.fits")


def test_reader_gives_rows_and_keywords():
    a = read_aspsol(ASPSOL_FILE)
    assert a.rows.shape[1] == len(ASPSOL_COLUMNS) == 7 and a.rows.shape[0] > 700
    assert a.tstart == 300000000.5 and a.ra_nom == 83.8221 and a.dec_nom == -5.3911 and a.roll_nom == 250.37
    assert np.all(np.diff(a.rows[:, 0]) > 0)
    assert abs(a.rows[0, 0] - (a.tstart - 1.0)) < 1e-6


def test_config_takes_the_files_pointing():
    a = read_aspsol(ASPSOL_FILE)
    c = apply_to_config(default_config(), a)
    assert c.dither == DITHER["FILE"] == 2
    assert (c.ra_nom, c.dec_nom, c.roll_nom) == (a.ra_nom, a.dec_nom, a.roll_nom)


def test_fixture_covers_every_photon():
    """The reference dithered every fixture photon (none past the table) and
    moved the detector by the file's dy, dz and dtheta."""
    for name in ("aspsol_scatter", "aspsol_hrci"):
        z = np.load(os.path.join(GOLDEN, f"trace_{name}.npz"))
        assert (z["used"][:, 1] >= 0).all()
        dd = z["det_dither"]
        assert np.abs(dd[0]).max() > 0.01 and np.abs(dd[1]).max() > 0.01 and 0 < np.abs(dd[2]).max() < 1e-4


def test_non_aspsol_file_is_refused(tmp_path):
    with pytest.raises(ValueError, match="ASPSOL"):
        read_aspsol(os.path.join(GOLDEN, "acis_fef_synthetic.fits"))
