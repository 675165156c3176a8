"""The SAOSAC source reader (host code) against the reference's SAOSAC
source reading the same synthetic ray files in batches, fed the same
per-row uniforms (tests/golden/saosac.npz): energies, positions,
directions, times relative to the batch before, vignetting flags (with the
flag a dropped row passes on) and mirror shells, exactly."""
import os

import numpy as np
import pytest

from marx_gb300 import workloads as W
from marx_gb300.saosac import SaosacFile

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("tag,fname", [("synthetic", "saosac_synthetic.fits"), ("notime", "saosac_notime.fits")])
def test_reader_matches_reference_batches(tag, fname):
    from marx_gb300.build import build
    build()
    z = np.load(os.path.join(GOLDEN, "saosac.npz"))
    cap = W.plain_hetg(parity=True).cfg.hrma_cap_x
    s = SaosacFile(os.path.join(GOLDEN, fname), cap)
    assert s.rows == 3000
    for b, m in enumerate((1000, 1000, 1500)):
        q = s.read(m, u=z["U"])
        assert q.n == int(z[f"{tag}_{b}_n"])
        for col in ("energy", "x", "p", "arrival_time", "flags"):
            assert np.array_equal(getattr(q, col), z[f"{tag}_{b}_{col}"]), (b, col)
        assert np.array_equal(q.mirror_shell.astype(np.int64), z[f"{tag}_{b}_mirror_shell"].astype(np.int64))
    assert s.read(10, u=z["U"]) is None
    s.close()


def test_reader_rejects_files_without_the_table(tmp_path):
    from marx_gb300.build import build
    build()
    p = tmp_path / "x.fits"
    p.write_bytes(b"SIMPLE  =                    T" + b" " * (2880 - 30))
    with pytest.raises(RuntimeError, match="RAYTRACE"):
        SaosacFile(str(p), 10000.0)
