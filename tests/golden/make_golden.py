"""Generate the golden fixtures from the reference MARX library itself.

    python tests/golden/make_golden.py

Needs the reference sources (MARX_REFERENCE_ROOT, default /root/reference);
oracle/Makefile compiles them in place into oracle/_ref.  Writes:

  trace_<workload>.npz   per-photon parity fixtures: seeded inputs, the
                         pre-drawn variates handed to the reference's stage
                         functions, and every output column the reference
                         produced (positions, directions, flags, shell,
                         order, chip, pixels, dither state).
  stats_<workload>.npz   seeded statistical fixtures from the reference's own
                         generator: encircled-energy curve, chip/pixel and
                         order histograms, survivor fractions.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from marx_gb300 import workloads as W  # noqa: E402
from marx_gb300.photons import predraw_variates  # noqa: E402
from oracle.bindings import Reference  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
N_TRACE = 1000
N_STATS = 200_000
EE_RADII = np.array([0.0025, 0.005, 0.01, 0.02, 0.04, 0.08, 0.16, 0.32, 0.64, 1.28])   # mm


def summarize(q, w):
    """Statistics compared against seeded GPU runs."""
    good = (q.flags & 0xFF) == 0
    out = {"good_fraction": np.array(good.mean()), "n": np.array(q.n)}
    if q.n and good.any():
        if w.cfg.grating == 0:
            # encircled energy about the detected centroid, detector plane (x = focal plane)
            y, z = q.x[1][good], q.x[2][good]
            r = np.hypot(y - np.median(y), z - np.median(z))
            out["ee_radii"] = EE_RADII
            out["ee"] = np.array([(r <= a).mean() for a in EE_RADII])
            out["radius_sample"] = np.sort(r)[:: max(1, len(r) // 5000)]
        else:
            orders = q.order[good].astype(int)
            out["order_hist"] = np.bincount(orders + 11, minlength=23)
        out["ccd_hist"] = np.bincount(q.ccd_num[good].astype(int) + 1, minlength=11)
    return out


def main():
    for name, make in W.PLAIN.items():
        w = make(parity=True)
        # per-photon parity fixture
        ph = w.photons(N_TRACE, seed=w.seed + 1)
        U, N = predraw_variates(N_TRACE, seed=w.seed + 2)
        ref = Reference(w.cfg)
        q, used, bad = ref.trace_slots(ph, U, N)
        assert bad == 0, "reference ran past its variate slots"
        np.savez_compressed(
            os.path.join(HERE, f"trace_{name}.npz"),
            energy=ph.energy, p_in=ph.p, arrival_time=ph.arrival_time, U=U, N=N,
            x=q.x, p=q.p, flags=q.flags, mirror_shell=q.mirror_shell, order=q.order, ccd_num=q.ccd_num,
            y_pixel=q.y_pixel, z_pixel=q.z_pixel, dither_state=q.dither_state, used=used)
        # statistical fixture with the reference's own generator
        ref_n = Reference(w.cfg, native=True, seed=w.seed)
        ph = w.photons(N_STATS, seed=w.seed + 3)
        q, secs = ref_n.trace_batch(ph)
        s = summarize(q, w)
        s["seconds"] = np.array(secs)
        np.savez_compressed(os.path.join(HERE, f"stats_{name}.npz"), **s)
        print(name, "good fraction", float(s["good_fraction"]), f"reference {N_STATS / secs:.3g} photons/s")


if __name__ == "__main__":
    main()
