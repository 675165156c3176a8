"""Shared helpers for the parity tests."""
import os

import numpy as np

from marx_gb300 import workloads as W
from marx_gb300.photons import PhotonList, NUM_U, NUM_N

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Tolerances of the parity contract: positions within 1e-9 mm; directions
# (unit vectors) within 1e-12; chip, pixel, order, shell and flags exact.
X_TOL_MM = 1e-9
P_TOL = 1e-12


def pad_slots(U, N):
    """Slot arrays widened to the current slot count (NUM_U, NUM_N).  Fixtures
    written before the LETG and HRC windows existed hold 16 uniforms and 8
    normals per photon; the stages they exercise read no slot beyond those."""
    n = U.shape[1]
    if U.shape[0] < NUM_U:
        U = np.vstack([U, np.full((NUM_U - U.shape[0], n), 0.5)])
    if N.shape[0] < NUM_N:
        N = np.vstack([N, np.zeros((NUM_N - N.shape[0], n))])
    return np.ascontiguousarray(U), np.ascontiguousarray(N)


def load_trace_fixture(name):
    z = np.load(os.path.join(GOLDEN, f"trace_{name}.npz"))
    w = W.ALL[name](parity=True)
    ph = PhotonList.from_inputs(z["energy"], z["p_in"], z["arrival_time"])
    U, N = pad_slots(z["U"], z["N"])
    return w, ph, U, N, z


def compare(q, ref, exact_fields=("flags", "mirror_shell", "order", "ccd_num", "y_pixel", "z_pixel", "dither_state")):
    """Returns a dict of mismatch counts / max deviations between two photon lists
    (ref may be a PhotonList or an npz with the same column names)."""
    g = lambda o, k: getattr(o, k) if hasattr(o, k) else o[k]
    out = {"dx": float(np.abs(q.x - g(ref, "x")).max()) if q.n else 0.0,
           "dp": float(np.abs(q.p - g(ref, "p")).max()) if q.n else 0.0}
    for k in exact_fields:
        out[k] = int(np.sum(g(q, k) != g(ref, k)))
    return out


# Dispersed spectra: equal-probability bins per (arm, order) histogram.
DISPERSED_BINS = 20


def dispersed_groups(q, cfg, orders=range(-3, 4)):
    """The detected photons' focal-plane coordinate along the dispersion
    direction of their grating arm, per arm and order: {"<arm>_<order>":
    values (mm)}.  The grating stage turns each photon by -theta (its
    shell's dispersion angle, plus LETG_ACIS_dTheta for the LETG on an
    ACIS detector) into the facet frame, where the grating's lines run
    along z and the dispersion along y (diffract.c:690-740, :1013), so the
    dispersion coordinate is y cos(theta) + z sin(theta).  HETG arms: MEG
    (shells 1 and 3), HEG (shells 4 and 6); the LETG has one arm."""
    good = ((q.flags & 0xFF) == 0) & (q.ccd_num >= 0)
    shell = q.mirror_shell.astype(int)
    if cfg.grating == 1:
        theta = np.asarray(cfg.hetg_theta[:])[shell]
        arm = np.where(shell < 2, "meg", "heg")
    else:
        theta = np.asarray(cfg.letg_theta[:])[shell] + (cfg.letg_acis_dtheta if cfg.detector in (1, 2) else 0.0)
        arm = np.full(q.n, "leg")
    th = np.deg2rad(theta)
    u = q.x[1] * np.cos(th) + q.x[2] * np.sin(th)
    out = {}
    for a in np.unique(arm):
        for m in orders:
            sel = good & (arm == a) & (q.order.astype(int) == m)
            out[f"{a}_{m}"] = u[sel]
    return out


EXTRA_FIELDS = ("support_orders", "pulse_height", "u_pixel", "v_pixel", "detector_region")


def assert_parity(q, ref, where="", pixel_ulps=0):
    """The parity contract.  pixel_ulps > 0 allows the single-precision chip
    pixels to differ by that many float steps where the FP64 positions
    behind them differ in their last bits (well inside the 1e-9 mm position
    tolerance) and round to neighbouring floats; the whole pixel
    (floor of y_pixel, z_pixel) must still be equal."""
    keys = getattr(ref, "files", None) or [k for k in EXTRA_FIELDS if hasattr(ref, k)]
    extra = tuple(k for k in EXTRA_FIELDS if k in keys and hasattr(q, k))
    exact = ("flags", "mirror_shell", "order", "ccd_num", "dither_state") + extra
    if not pixel_ulps:
        exact += ("y_pixel", "z_pixel")
    r = compare(q, ref, exact_fields=exact)
    assert r["dx"] <= X_TOL_MM, (where, r)
    assert r["dp"] <= P_TOL, (where, r)
    bad = {k: v for k, v in r.items() if k not in ("dx", "dp") and v}
    assert not bad, (where, r)
    if pixel_ulps:
        g = lambda o, k: getattr(o, k) if hasattr(o, k) else o[k]  # noqa: E731
        for k in ("y_pixel", "z_pixel"):
            a, b = g(q, k), g(ref, k)
            steps = np.abs(a.view(np.int32).astype(np.int64) - b.view(np.int32).astype(np.int64))
            assert int(steps.max(initial=0)) <= pixel_ulps, (where, k, int(steps.max()))
            assert np.array_equal(np.floor(a), np.floor(b)), (where, k, "whole pixel")
            # a last-bit flip needs a float rounding boundary between the two
            # FP64 positions: rare
            assert int((steps != 0).sum()) <= max(8, a.size // 200_000), (where, k, int((steps != 0).sum()))
