"""Shared helpers for the parity tests."""
import os

import numpy as np

from marx_gb300 import workloads as W
from marx_gb300.photons import PhotonList

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Tolerances of the parity contract: positions within 1e-9 mm; directions
# (unit vectors) within 1e-12; chip, pixel, order, shell and flags exact.
X_TOL_MM = 1e-9
P_TOL = 1e-12


def load_trace_fixture(name):
    z = np.load(os.path.join(GOLDEN, f"trace_{name}.npz"))
    w = W.PLAIN[name](parity=True)
    ph = PhotonList.from_inputs(z["energy"], z["p_in"], z["arrival_time"])
    return w, ph, z["U"], z["N"], z


def compare(q, ref, exact_fields=("flags", "mirror_shell", "order", "ccd_num", "y_pixel", "z_pixel", "dither_state")):
    """Returns a dict of mismatch counts / max deviations between two photon lists
    (ref may be a PhotonList or an npz with the same column names)."""
    g = lambda o, k: getattr(o, k) if hasattr(o, k) else o[k]
    out = {"dx": float(np.abs(q.x - g(ref, "x")).max()) if q.n else 0.0,
           "dp": float(np.abs(q.p - g(ref, "p")).max()) if q.n else 0.0}
    for k in exact_fields:
        out[k] = int(np.sum(g(q, k) != g(ref, k)))
    return out


def assert_parity(q, ref, where=""):
    r = compare(q, ref)
    assert r["dx"] <= X_TOL_MM, (where, r)
    assert r["dp"] <= P_TOL, (where, r)
    bad = {k: v for k, v in r.items() if k not in ("dx", "dp") and v}
    assert not bad, (where, r)
