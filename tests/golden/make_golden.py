"""Generate the golden fixtures from the reference MARX library itself.

    python tests/golden/make_golden.py [workload ...]

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
  dat_<workload>.npz     the reference's output files (marx_write_photons)
                         for the photons of trace_<workload>.npz, written
                         then appended to (--dat).
  sources.npz            energies and directions of the reference's source
                         models (POINT, GAUSS, BETA, DISK, LINE; FLAT and
                         FILE spectra) for the engine's source uniforms
                         (--sources).
  diff_rays.npz          focal-plane positions of the differentiable form's
                         rays traced by the reference's mirror stage, at
                         theta = 0 and at the workload's perturbation written
                         into a copy of the HRMA geometry file, for an ideal
                         and a reflecting (no blur, no scattering) mirror.
"""
from __future__ import annotations

import os
import shutil
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from marx_gb300 import workloads as W  # noqa: E402
from marx_gb300.photons import predraw_variates  # noqa: E402
from oracle.bindings import Reference, Oracle, REF_ROOT  # noqa: E402
from marx_gb300.diff import diff_workload, diff_mirror_config, source_direction, NPARAM  # noqa: E402
from marx_gb300.photons import PhotonList, NUM_U, NUM_N  # noqa: E402

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
            if w.cfg.grating == 2:      # LETG: orders -25..25, and the fine support orders
                out["order_hist"] = np.bincount(orders + 25, minlength=51)
                out["fine_hist"] = np.bincount(q.support_orders[0][good].astype(int) + 9, minlength=19)
            else:
                out["order_hist"] = np.bincount(orders + 11, minlength=23)
        out["ccd_hist"] = np.bincount(q.ccd_num[good].astype(int) + 1, minlength=11)
        if w.cfg.detector >= 3:     # HRC: pulse heights in bins of 16, shield regions
            out["pha_hist"] = np.bincount(q.pulse_height[good].astype(int) // 16, minlength=40)[:40]
            if w.cfg.detector == 4:
                out["region_hist"] = np.bincount(q.detector_region[good].astype(int), minlength=4)
    return out


def main(names=None):
    for name, make in W.ALL.items():
        if names and name not in names:
            continue
        w = make(parity=True)
        # per-photon parity fixture
        ph = w.photons(N_TRACE, seed=w.seed + 1)
        U, N = predraw_variates(N_TRACE, seed=w.seed + 2)
        ref = Reference(w.cfg)
        q, used, bad = ref.trace_slots(ph, U, N)
        assert bad == 0, "reference ran past its variate slots"
        extra = {}
        if w.cfg.grating == 2:
            extra["support_orders"] = q.support_orders
        if w.cfg.detector >= 3:
            extra.update(pulse_height=q.pulse_height, detector_region=q.detector_region)
            if w.cfg.detector == 4:
                extra.update(u_pixel=q.u_pixel, v_pixel=q.v_pixel)
        np.savez_compressed(
            os.path.join(HERE, f"trace_{name}.npz"),
            energy=ph.energy, p_in=ph.p, arrival_time=ph.arrival_time, U=U, N=N,
            x=q.x, p=q.p, flags=q.flags, mirror_shell=q.mirror_shell, order=q.order, ccd_num=q.ccd_num,
            y_pixel=q.y_pixel, z_pixel=q.z_pixel, dither_state=q.dither_state, used=used, **extra)
        # statistical fixture with the reference's own generator
        ref_n = Reference(w.cfg, native=True, seed=w.seed)
        ph = w.photons(N_STATS, seed=w.seed + 3)
        q, secs = ref_n.trace_batch(ph)
        s = summarize(q, w)
        s["seconds"] = np.array(secs)
        np.savez_compressed(os.path.join(HERE, f"stats_{name}.npz"), **s)
        print(name, "good fraction", float(s["good_fraction"]), f"reference {N_STATS / secs:.3g} photons/s")


DAT_WORKLOADS = ("plain_scatter", "letg_hrcs")


def dat_fixture(name):
    """The reference's own writer (marx_write_photons) on a trace fixture's
    output photons: a new output directory, then a second batch appended.
    Runs in a process of its own: the reference keeps each file's row count
    in a static that no later directory resets."""
    from helpers import load_trace_fixture
    from marx_gb300 import output as O
    w, ph, U, N, z = load_trace_fixture(name)
    q = ph.copy()
    for k in z.files:
        if hasattr(q, k) and k != "energy":
            getattr(q, k)[...] = z[k]
    h = O.history(w.cfg)
    ref = Reference(w.cfg)
    d = tempfile.mkdtemp()
    try:
        ref.write_photons(q, h, O.ALL, d, new=True, total_time=12.5)
        ref.write_photons(q, h, O.ALL, d, new=False, total_time=100.0)
        files = {f: np.frombuffer(open(os.path.join(d, f), "rb").read(), dtype=np.uint8) for f in os.listdir(d)}
    finally:
        shutil.rmtree(d)
    np.savez_compressed(os.path.join(HERE, f"dat_{name}.npz"), history=np.array(h), **files)
    print(name, "output files", len(files))


N_SRC = 2000
# source models of the sources fixture: (name, SourceType, parameter overrides, mx_source param)
SOURCE_CASES = (
    ("point", "POINT", {}, ()),
    ("gauss", "GAUSS", {"S-GaussSigma": "20.0"}, (20.0,)),
    ("beta", "BETA", {"S-BetaCoreRadius": "12.5", "S-BetaBeta": "0.8"}, (12.5, 0.8)),
    ("disk", "DISK", {"S-DiskTheta0": "15.0", "S-DiskTheta1": "75.0"}, (15.0, 75.0)),
    ("line", "LINE", {"S-LinePhi": "30.0", "S-LineTheta": "300.0"}, (30.0, 300.0)),
    ("gauss_file", "GAUSS", {"S-GaussSigma": "5.0"}, (5.0,)),
)


def source_spectrum():
    """A smooth absorbed power law on 0.2-9 keV, 400 rows: the FILE
    spectrum of the gauss_file case."""
    e = np.linspace(0.2, 9.0, 400)
    f = e ** -1.7 * np.exp(-0.3 * e ** (-8.0 / 3.0))
    return e, f


def sources_fixture():
    """The reference's source models, one create_photons call per photon,
    with the Philox source-domain uniforms the engine draws for the same
    tags (draw k of tag i in slot k)."""
    w = W.plain_onaxis(parity=True)
    oracle = Oracle(w.cfg)
    seed = 4321
    tags = np.arange(N_SRC, dtype=np.uint32)
    U = np.array([[oracle.source_uniform(seed, int(i), k) for i in tags] for k in range(4)])
    out = {"seed": np.array(seed), "n": np.array(N_SRC), "U": U}
    e_spec, f_spec = source_spectrum()
    out["spectrum_energy"], out["spectrum_flux"] = e_spec, f_spec
    tmp = tempfile.mkdtemp()
    try:
        spec_file = os.path.join(tmp, "spectrum.dat")
        with open(spec_file, "w") as fh:
            for a, b in zip(e_spec, f_spec):
                fh.write(f"{float(a)!r} {float(b)!r}\n")
        for name, kind, over, param in SOURCE_CASES:
            par = {"SourceType": kind, "SourceRA": "250.25", "SourceDEC": "-53.73", "MinEnergy": "0.5",
                   "MaxEnergy": "7.0", "SpectrumType": "FILE" if name.endswith("_file") else "FLAT",
                   "SpectrumFile": spec_file, **over}
            ref = Reference(w.cfg, extra_par=par)
            p0, e, p = ref.source_photons(N_SRC, U)
            out[f"{name}_src"] = p0
            out[f"{name}_param"] = np.array(param, dtype=np.float64)
            out[f"{name}_energy"] = e
            out[f"{name}_p"] = p
            print("source", name, p0, e[:2])
    finally:
        shutil.rmtree(tmp)
    np.savez_compressed(os.path.join(HERE, "sources.npz"), **out)


N_DIFF = 4000
RDB = "EKCHDOS06.rdb"
SHELL_OF = {"1": 0, "3": 1, "4": 2, "6": 3}


def perturbed_datadir(theta, where: str) -> str:
    """A MARX data directory whose HRMA geometry file has theta added to
    az_mis, el_mis (arcsec -> degrees) and x0, y0 (um -> mm) of both rows of
    every shell; every other file is a link to the reference's own."""
    src = os.path.join(REF_ROOT, "marx", "data")
    for e in os.listdir(src):
        if e != "hrma":
            os.symlink(os.path.join(src, e), os.path.join(where, e))
    os.makedirs(os.path.join(where, "hrma"))
    for e in os.listdir(os.path.join(src, "hrma")):
        if e != RDB:
            os.symlink(os.path.join(src, "hrma", e), os.path.join(where, "hrma", e))
    lines = open(os.path.join(src, "hrma", RDB)).read().split("\n")
    cols = None
    out = []
    for ln in lines:
        f = ln.split("\t")
        if cols is None and f and f[0] == "mirror":
            cols = {c: k for k, c in enumerate(f)}
        elif cols is not None and f and f[0][:1] in "ph" and f[0][1:] in SHELL_OF:
            s = SHELL_OF[f[0][1:]]
            add = {"az_mis": theta[4 * s] / 3600.0, "el_mis": theta[4 * s + 1] / 3600.0,
                   "x0": theta[4 * s + 2] * 1e-3, "y0": theta[4 * s + 3] * 1e-3}
            for c, d in add.items():
                f[cols[c]] = repr(float(float(f[cols[c]]) + float(d)))
            ln = "\t".join(f)
        out.append(ln)
    with open(os.path.join(where, "hrma", RDB), "w") as fh:
        fh.write("\n".join(out))
    return where


def diff_rays():
    """The reference's mirror stage on the weighted rays' aperture points:
    each photon gets the Philox variates of its tag, so it picks the shell,
    radius and azimuth the engine's ray of that tag picks."""
    w = diff_workload(n_rays=N_DIFF)
    oracle = Oracle(diff_mirror_config(ideal=True))
    tags = np.arange(N_DIFF, dtype=np.uint32)
    U = np.array([[oracle.philox_uniform(w.cfg.seed, int(i), k) for i in tags] for k in range(NUM_U)])
    N = np.array([[oracle.philox_normal(w.cfg.seed, int(i), k) for i in tags] for k in range(NUM_N)])
    out = {"seed": np.array(w.cfg.seed), "n": np.array(N_DIFF), "energy": np.array(w.cfg.energy),
           "src": np.array([w.cfg.src_y, w.cfg.src_z])}
    thetas = {"zero": np.zeros(NPARAM), "true": w.theta_true}
    for mname, ideal in (("ideal", True), ("reflect", False)):
        cfg = diff_mirror_config(ideal=ideal)
        cfg.use_blur = 0
        cfg.use_wfold = 0
        for tname, theta in thetas.items():
            tmp = tempfile.mkdtemp(prefix="mxdiff")
            try:
                ref = Reference(cfg, datadir=perturbed_datadir(theta, tmp))
                p0 = source_direction(w.cfg.src_y + theta[16], w.cfg.src_z + theta[17])
                ph = PhotonList.from_inputs(np.full(N_DIFF, w.cfg.energy), np.repeat(p0[:, None], N_DIFF, 1),
                                            np.zeros(N_DIFF))
                ph.tag[:] = tags
                q, used, bad = ref.trace_slots(ph, U, N, stages=2)
                assert bad == 0
            finally:
                shutil.rmtree(tmp)
            hit = (q.flags & 0xFF) == 0
            t = -q.x[0] / q.p[0]
            out[f"{mname}_{tname}_y"] = np.where(hit, q.x[1] + t * q.p[1], np.nan)
            out[f"{mname}_{tname}_z"] = np.where(hit, q.x[2] + t * q.p[2], np.nan)
            out[f"{mname}_{tname}_theta"] = theta
            print(mname, tname, "reflected", hit.mean())
    np.savez_compressed(os.path.join(HERE, "diff_rays.npz"), **out)


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(HERE))
    names = [a for a in sys.argv[1:] if not a.startswith("-")]
    if "--diff" in sys.argv:
        diff_rays()
    elif "--sources" in sys.argv:
        sources_fixture()
    elif "--dat" in sys.argv:
        if names:
            dat_fixture(names[0])
        else:
            import subprocess
            for n in DAT_WORKLOADS:
                subprocess.run([sys.executable, __file__, "--dat", n], check=True)
    elif names:
        main(names)
    else:
        main()
        diff_rays()
