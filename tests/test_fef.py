"""The ACIS FEF on the CPU: the pack reads the FEF file's FUNCTION table as
the reference's read_fef_file does, and the engine builds its regions (no
GPU: mx_validate_config)."""
import os

import numpy as np

from marx_gb300.caldb.pack import DEFAULT_PACK, pack_with_fef, read_contam, read_fef, read_pack
from marx_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FEF_FILE = os.path.join(GOLDEN, "acis_fef_synthetic.fits")
CONTAM_FILE = os.path.join(GOLDEN, "acis_contam_synthetic.fits")


def test_fef_sections():
    S = read_fef(FEF_FILE)
    rows, vals = S["acis/fef/rows"], S["acis/fef/vals"]
    assert rows.shape == (800, 6) and vals.shape == (800, 2 + 3 * 3)
    assert set(rows[:, 0]) == set(range(10))
    # rows of one region are consecutive, energies and channels ascending
    for reg in np.unique(rows[:, 5]):
        m = np.nonzero(rows[:, 5] == reg)[0]
        assert np.all(np.diff(m) == 1)
        assert np.all(np.diff(vals[m, 0]) > 0) and np.all(np.diff(vals[m, 1]) > 0)
    # negative shoulders on the BI chips only
    neg = vals[:, 2 + 3 * 1 + 2] < 0
    assert set(rows[neg, 0]) == {5, 7}


def test_pack_with_fef_builds_the_engine_model(tmp_path):
    from marx_gb300._native import validate_config
    out = str(tmp_path / "fef.mxpack")
    pack_with_fef(DEFAULT_PACK, FEF_FILE, out)
    S = read_pack(out)
    assert "acis/fef/rows" in S and "hrma/rdb" in S
    for name in ("plain_scatter", "plain_hetg"):
        assert validate_config(W.ALL[name](parity=True).cfg, pack=out) is None
    # a malformed FEF (a region not on the 32-pixel grid) is refused
    S["acis/fef/rows"] = S["acis/fef/rows"].copy()
    S["acis/fef/rows"][0, 2] = 500
    from marx_gb300.caldb.pack import write_pack
    bad = str(tmp_path / "bad.mxpack")
    write_pack(bad, S)
    assert "multiple of 32" in (validate_config(W.ALL["plain_scatter"](parity=True).cfg, pack=bad) or "")


def test_contam_sections_and_model(tmp_path):
    """The contamination tables per chip (two layers; an fxy map on the BI
    chips), and an engine model with the QE acceptance (DetIdeal = no)."""
    from marx_gb300._native import validate_config
    S = read_contam(CONTAM_FILE)
    for ccd in range(10):
        assert S[f"acis/contam{ccd}/rows"].shape == (2, 3)
        assert (f"acis/contam{ccd}/fxy" in S) == (ccd in (5, 7))
    out = str(tmp_path / "qe.mxpack")
    pack_with_fef(DEFAULT_PACK, FEF_FILE, out, contam_path=CONTAM_FILE)
    for name in ("plain_scatter", "plain_hetg"):
        cfg = W.ALL[name](parity=True).cfg
        cfg.det_ideal = 0
        assert validate_config(cfg, pack=out) is None
    # a layer that is not component 0 is refused, as the reference does
    T = read_pack(out)
    T["acis/contam0/rows"] = T["acis/contam0/rows"].copy()
    T["acis/contam0/rows"][1, 0] = 1
    from marx_gb300.caldb.pack import write_pack
    bad = str(tmp_path / "bad.mxpack")
    write_pack(bad, T)
    cfg = W.ALL["plain_scatter"](parity=True).cfg
    cfg.det_ideal = 0
    assert "COMPONENT=0" in (validate_config(cfg, pack=bad) or "")
