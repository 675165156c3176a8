"""DitherModel = FILE: the aspect solution the reference's dither module
reads (init_aspsol_dither, marx/libsrc/dither.c:438-500).

The ASPSOL binary table gives, per row, the time (s), the pointing ra, dec
and roll (degrees), the detector's offsets dy, dz (mm) and its rotation
dtheta (degrees); its header carries RA_NOM, DEC_NOM, ROLL_NOM (degrees)
and TSTART (s).  ``read_aspsol`` reads those as doubles, as
jdfits_simple_d_read_btable does; the engine converts the rows and keeps
them on the device (``Engine.set_aspect_solution``, mx_set_aspect_solution).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .caldb.pack import read_fits_bintables
from .config import DITHER, MxConfig

ASPSOL_COLUMNS = ("time", "ra", "dec", "roll", "dy", "dz", "dtheta")


@dataclass
class AspectSolution:
    rows: np.ndarray          # (n, 7) float64 in ASPSOL_COLUMNS order
    ra_nom: float
    dec_nom: float
    roll_nom: float
    tstart: float


def read_aspsol(path: str) -> AspectSolution:
    """The ASPSOL extension of `path` (column names matched without regard
    to case, as the reference's table reader does)."""
    for hdr, cols in read_fits_bintables(path):
        if hdr.get("EXTNAME", "").strip().upper() != "ASPSOL":
            continue
        by = {k.lower(): v for k, v in cols.items()}
        missing = [c for c in ASPSOL_COLUMNS if c not in by]
        if missing:
            raise ValueError(f"{path}: ASPSOL table lacks {missing}")
        keys = {}
        for k in ("RA_NOM", "DEC_NOM", "ROLL_NOM", "TSTART"):
            if k not in hdr:
                raise ValueError(f"Unable to find keyword {k} in ASPSOL file {path}")
            keys[k] = float(hdr[k])
        rows = np.stack([np.asarray(by[c], dtype=np.float64).reshape(-1) for c in ASPSOL_COLUMNS], axis=1)
        if len(rows) == 0:
            raise ValueError(f"{path}: ASPSOL file contains no data")
        return AspectSolution(np.ascontiguousarray(rows), keys["RA_NOM"], keys["DEC_NOM"], keys["ROLL_NOM"],
                              keys["TSTART"])
    raise ValueError(f"Unable to open a proper ASPSOL file called {path}")


def apply_to_config(cfg: MxConfig, asp: AspectSolution) -> MxConfig:
    """DitherModel FILE with the file's nominal pointing, which replaces the
    parameter file's RA_Nom, Dec_Nom and Roll_Nom (init_aspsol_dither)."""
    cfg.dither = DITHER["FILE"]
    cfg.ra_nom, cfg.dec_nom, cfg.roll_nom = asp.ra_nom, asp.dec_nom, asp.roll_nom
    return cfg
