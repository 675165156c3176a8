"""Generate the golden fixtures from the reference MARX library itself.

    python tests/golden/make_golden.py [workload ...]

Needs the reference sources (MARX_REFERENCE_ROOT, else the checkout
oracle/Makefile names); oracle/Makefile compiles them in place into
oracle/_ref.  Writes:

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
  events_<case>.npz      the reference's marx2fits program (oracle/Makefile
                         target m2f) run on a synthetic output directory:
                         the event columns it read, the facet geometry, and
                         CHIPX/CHIPY, EXPNO, FLTGRADE/GRADE, TDETX/TDETY,
                         DETX/DETY and X/Y of its FITS event list for each
                         pixel adjustment (--events).
  acis_fef_synthetic.fits  a synthetic ACIS FEF (the real one is not in the
                         reference checkout): 10 chips x 4 regions x 20
                         energies, three gaussians per row (main peak, a
                         shoulder that is negative on the BI chips 5 and 7,
                         a low-channel tail) (--fef).
  trace_fef_<workload>.npz, stats_fef_<workload>.npz
                         the trace and statistics fixtures of a workload
                         with the reference's ACIS detector reading that FEF
                         (pulse height and PI) (--fef).
  aspsol_synthetic.fits, trace_aspsol_<case>.npz
                         a synthetic ASPSOL aspect solution and the trace of
                         a workload's photons by the reference with
                         DitherModel = FILE reading it (sky and detector
                         dither state recorded) (--aspsol).
  dispersed_<workload>.npz
                         dispersed spectra of the reference's own seeded
                         run of 1e6 photons through the HETG or LETG: the
                         detected photons' focal-plane coordinate along the
                         dispersion direction of their grating arm, per arm
                         and order (-3..3), as samples and histograms
                         (--dispersed).
  saosac_synthetic.fits, saosac_notime.fits, saosac.npz
                         synthetic SAO raytrace files (RAYTRACE tables of
                         rays on the four shells' exit annuli toward the
                         focus, weights, with and without RT_TIME) and the
                         photons the reference's SAOSAC source makes of them
                         in batches, fed per-row uniforms (--saosac).
  diff_fd_reference.npz  central finite differences of the reference itself
                         for the differentiable form: 2e5 rays (Philox
                         variates of their tags, so common random numbers
                         at every step) through the reference's ideal mirror
                         with each of the 18 parameters moved by +-h in the
                         HRMA geometry file (and the source direction),
                         imaged with the engine's splat; the MSE to a target
                         image and the 18-gradient, at theta_true and at a
                         random theta (--diff-fd).
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
    ("image", "IMAGE", {}, (0.6 / 3600.0, 0.6 / 3600.0)),   # S-ImageFile: source_image() as FITS
)


def source_image():
    """A 48 x 64 image for the IMAGE case: two Gaussian blobs on a floor,
    a block of empty pixels (flat runs in the cumulative distribution) and
    one bright pixel; 0.6 arcsec pixels."""
    ny, nx = 48, 64
    yy, xx = np.mgrid[0:ny, 0:nx].astype(np.float64)
    im = 50 * np.exp(-((xx - 20) ** 2 + (yy - 30) ** 2) / 18.0) + 20 * np.exp(-((xx - 45) ** 2 + (yy - 12) ** 2) / 40.0)
    im += 0.3
    im[5:15, 50:60] = 0.0
    im[40, 8] = 400.0
    return im.astype(np.float32), (0.6 / 3600.0, 0.6 / 3600.0)


def write_image_fits(path, im, scale):
    """A primary-HDU FITS image (BITPIX -32) with CDELT1/CDELT2."""
    ny, nx = im.shape
    cards = [("SIMPLE", "T"), ("BITPIX", "-32"), ("NAXIS", "2"), ("NAXIS1", str(nx)), ("NAXIS2", str(ny)),
             ("CDELT1", repr(-scale[0])), ("CDELT2", repr(scale[1]))]
    h = "".join(f"{k:<8}= {v:>20}" .ljust(80) for k, v in cards) + "END".ljust(80)
    h = h.ljust((len(h) + 2879) // 2880 * 2880)
    data = im.astype(">f4").tobytes()
    data += b"\0" * ((-len(data)) % 2880)
    with open(path, "wb") as f:
        f.write(h.encode("ascii") + data)


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
        img_file = os.path.join(tmp, "image.fits")
        im, scale = source_image()
        write_image_fits(img_file, im, scale)
        out["image"] = im
        out["image_scale"] = np.array(scale)
        for name, kind, over, param in SOURCE_CASES:
            par = {"SourceType": kind, "SourceRA": "250.25", "SourceDEC": "-53.73", "MinEnergy": "0.5",
                   "MaxEnergy": "7.0", "SpectrumType": "FILE" if name.endswith("_file") else "FLAT",
                   "SpectrumFile": spec_file, "S-ImageFile": img_file, **over}
            ref = Reference(w.cfg, extra_par=par)
            # an IMAGE source's st->p is left pointing to the sky (source.c:158-201);
            # its photons are drawn about the point source's direction of travel instead
            p0, e, p = ref.source_photons(N_SRC, U, direction=out.get("point_src") if kind == "IMAGE" else None)
            out[f"{name}_src"] = p0
            out[f"{name}_param"] = np.array(param, dtype=np.float64)
            out[f"{name}_energy"] = e
            out[f"{name}_p"] = p
            print("source", name, p0, e[:2])
    finally:
        shutil.rmtree(tmp)
    np.savez_compressed(os.path.join(HERE, "sources.npz"), **out)


# ----------------------------------------------------------- event lists --
# (workload whose configuration names the detector, marx2fits inputs)
EVENT_CASES = {
    "acis_i": dict(workload="plain_scatter", detector="ACIS-I", dithered=True, roll_nom=237.36968458476,
                   det_offset=(0.0, 0.0, 0.0), motion=False, focal=10070.0),
    "acis_s": dict(workload="plain_hetg", detector="ACIS-S", dithered=True, roll_nom=112.25,
                   det_offset=(0.2, -0.35, 0.15), motion=True, focal=10079.77),
    "acis_i_nodither": dict(workload="plain_onaxis", detector="ACIS-I", dithered=False, roll_nom=37.5,
                            det_offset=(0.0, 0.1, 0.0), motion=False, focal=10070.0),
    "hrc_i": dict(workload="plain_hrci", detector="HRC-I", dithered=True, roll_nom=10.0,
                  det_offset=(0.0, 0.0, 0.0), motion=False, focal=10070.0),
    "hrc_s": dict(workload="letg_hrcs", detector="HRC-S", dithered=True, roll_nom=300.0,
                  det_offset=(0.0, 0.1, -0.2), motion=False, focal=10070.0),
}
N_EVENTS = 4000
FRAME_TIME = 3.2 + 0.041          # marx.par ACIS_Exposure_Time + ACIS_Frame_Transfer_Time
PIXADJ_MODES = ("EXACT", "NONE", "RANDOMIZE", "EDSER")


def write_dat(path, name, typ, values):
    """One column file of a MARX output directory (marx/data/FORMAT.TXT)."""
    dt = {"E": ">f4", "J": ">i4", "I": ">i2", "A": ">i1"}[typ]
    v = np.asarray(values).astype(dt)
    hdr = bytearray(32)
    hdr[0:4] = bytes([0x83, 0x13, 0x89, 0x8D])
    hdr[4] = ord(typ)
    hdr[5:5 + len(name)] = name.encode()
    hdr[20:24] = len(v).to_bytes(4, "big")
    with open(path, "wb") as f:
        f.write(bytes(hdr) + v.tobytes())


def par_set(text, name, value):
    """Set the value field of one parameter line of a .par file."""
    out = []
    for line in text.splitlines():
        if line.split(",", 1)[0] == name:
            f = line.split(",")
            f[3] = value
            line = ",".join(f)
        out.append(line)
    return "\n".join(out) + "\n"


def synth_events(case, geom, seed):
    rng = np.random.default_rng(seed)
    n = N_EVENTS
    ids = geom[:, 0].astype(np.int64)
    ccd = ids[rng.integers(0, len(ids), n)]
    det = case["detector"]
    nx, ny = {"ACIS-I": (1024, 1024), "ACIS-S": (1024, 1024), "HRC-I": (16384, 16384),
              "HRC-S": (4096, 16456)}[det]
    xp = rng.uniform(0, nx, n)
    yp = rng.uniform(0, ny, n)
    # whole pixels and sub-pixel thirds, where floor and the grade split change
    m = rng.random(n) < 0.1
    xp[m] = np.floor(xp[m])
    m = rng.random(n) < 0.1
    yp[m] = np.floor(yp[m]) + rng.choice([1.0 / 3.0, 2.0 / 3.0, 0.5], int(m.sum()))
    t = np.sort(rng.uniform(0.0, n / 30.0 * FRAME_TIME, n)).astype(np.float32)
    arc = np.pi / (180.0 * 3600.0)
    ra = 8.0 * arc * np.sin(2 * np.pi * t / 1000.0) + rng.normal(0, 0.2 * arc, n)
    dec = 8.0 * arc * np.sin(2 * np.pi * t / 707.0) + rng.normal(0, 0.2 * arc, n)
    roll = np.deg2rad(case["roll_nom"]) + rng.normal(0, 1e-5, n)
    z = np.zeros(n)
    dy = rng.normal(0, 0.02, n) if case["motion"] else z
    dz = rng.normal(0, 0.02, n) if case["motion"] else z
    dth = rng.normal(0, 2e-4, n) if case["motion"] else z
    be = rng.uniform(0.2, 12.0, n)
    be[:20] = [0.0, 20.0, 0.3, 1.0, 2.0, 0.5, 5.0, 10.0, 1.5, 0.25] * 2   # table nodes and ends
    U = rng.random((3, n))
    U[:, :8] = [[0.0] * 8, [0.0] * 8, [0.999999] * 8]
    f = np.float32
    return dict(ccd=ccd.astype(np.int8), xpixel=xp.astype(f), ypixel=yp.astype(f), time=t,
                sky_ra=ra.astype(f), sky_dec=dec.astype(f), sky_roll=roll.astype(f), det_dy=dy.astype(f),
                det_dz=dz.astype(f), det_theta=dth.astype(f), b_energy=be.astype(f)), U


def run_marx2fits(case, ev, U, mode, workdir):
    """The reference's marx2fits on one synthetic output directory."""
    import subprocess
    from marx_gb300.caldb.pack import read_fits_bintables
    exe = os.path.join(ROOT, "oracle", "_ref", "marx2fits")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "m2f", f"REF={REF_ROOT}"], check=True)
    d = os.path.join(workdir, f"sim_{mode}")
    os.makedirs(d, exist_ok=True)
    n = len(ev["ccd"])
    acis = case["detector"].startswith("ACIS")
    z = np.zeros(n)
    cols = [("time.dat", "TIME", "E", ev["time"]), ("energy.dat", "ENERGY", "E", z + 1.0),
            ("b_energy.dat", "B_ENERGY", "E", ev["b_energy"]),
            ("xpos.dat", "XPOS", "E", z), ("ypos.dat", "YPOS", "E", z), ("zpos.dat", "ZPOS", "E", z),
            ("xcos.dat", "COSX", "E", z - 1.0), ("ycos.dat", "COSY", "E", z), ("zcos.dat", "COSZ", "E", z),
            ("pha.dat", "PHA", "I", z), ("detector.dat", "CCDID", "A", ev["ccd"]),
            ("xpixel.dat", "CHIPX", "E", ev["xpixel"]), ("ypixel.dat", "CHIPY", "E", ev["ypixel"]),
            ("mirror.dat", "MIRROR", "I", z), ("tag.dat", "TAG", "J", np.arange(n)),
            ("sky_ra.dat", "RA", "E", ev["sky_ra"]), ("sky_dec.dat", "DEC", "E", ev["sky_dec"]),
            ("sky_roll.dat", "ROLL", "E", ev["sky_roll"]), ("det_dy.dat", "DET_DY", "E", ev["det_dy"]),
            ("det_dz.dat", "DET_DZ", "E", ev["det_dz"]), ("det_theta.dat", "DET_THETA", "E", ev["det_theta"])]
    if case["detector"] == "HRC-S":
        cols += [("hrc_u.dat", "U", "E", z), ("hrc_v.dat", "V", "E", z)]
    for fn, name, typ, v in cols:
        write_dat(os.path.join(d, fn), name, typ, v)
    par = open(os.path.join(REF_ROOT, "marx", "par", "marx.par")).read()
    for k, v in (("DetectorType", f'"{case["detector"]}"'), ("GratingType", '"NONE"'),
                 ("DitherModel", '"INTERNAL"' if case["dithered"] else '"NONE"'),
                 ("FocalLength", repr(case["focal"])), ("DetOffsetX", repr(case["det_offset"][0])),
                 ("DetOffsetY", repr(case["det_offset"][1])), ("DetOffsetZ", repr(case["det_offset"][2])),
                 ("ACIS_Exposure_Time", "3.2"), ("ACIS_Frame_Transfer_Time", "0.041")):
        par = par_set(par, k, v)
    open(os.path.join(d, "marx.par"), "w").write(par)
    obs_t = {"ACIS-I": "acis_i_obs.par", "ACIS-S": "acis_s_obs.par", "HRC-I": "hrc_i_obs.par",
             "HRC-S": "hrc_s_obs.par"}[case["detector"]]
    obs = open(os.path.join(REF_ROOT, "marx", "data", "obs", obs_t)).read()
    # the values marx's write_obs_par learns into the template (marx.c:1152-1180)
    for k, v in (("EXPOSURE", 1000.0), ("ra_nom", 250.2), ("dec_nom", -53.75), ("roll_nom", case["roll_nom"]),
                 ("tstart", 0.0), ("tstop", 1000.0), ("sim_x", 0.0), ("sim_y", 0.0), ("sim_z", 0.0)):
        obs = par_set(obs, k, repr(v))
    open(os.path.join(d, "obs.par"), "w").write(obs)
    # the uniforms in the order marx2fits draws them
    padj = mode if (acis or mode != "EDSER") else "RANDOMIZE"
    seq = []
    for k in range(n):
        if acis:
            seq.append(U[0, k])
        if padj == "RANDOMIZE":
            seq += [U[1, k], U[2, k]]
    ufile = os.path.join(workdir, f"u_{mode}.bin")
    np.asarray(seq, dtype=np.float64).tofile(ufile)
    out = os.path.join(workdir, f"evt_{mode}.fits")
    env = dict(os.environ, MARX_DATA_DIR=os.path.join(REF_ROOT, "marx", "data"), MXREF_UNIFORMS=ufile)
    r = subprocess.run([exe, f"--pixadj={mode}", d, out], env=env, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"marx2fits failed: {r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    drawn = [ln for ln in r.stderr.splitlines() if ln.startswith("mxref uniforms drawn:")]
    got = int(drawn[-1].split(":")[1]) if drawn else 0
    if got != len(seq):
        raise RuntimeError(f"marx2fits drew {got} uniforms, expected {len(seq)}")
    for hdr, c in read_fits_bintables(out):
        if hdr.get("EXTNAME") == "EVENTS":
            return c
    raise RuntimeError("no EVENTS table")


def events_fixture(name):
    """The reference's marx2fits on a synthetic event list (one process per
    case: the reference keeps detector state in statics)."""
    case = EVENT_CASES[name]
    w = W.ALL[case["workload"]]()
    ref = Reference(w.cfg)
    geom, tdet, fp = ref.detector_geometry(), ref.facet_tdet(), ref.fp_system()
    import zlib
    ev, U = synth_events(case, geom, seed=zlib.crc32(name.encode()))
    out = dict(geom=geom, tdet=tdet, fp=fp, uniforms=U, **ev)
    if case["detector"] == "HRC-I":
        # marx2fits cannot open an HRC-I run in this MARX: the detector set-up
        # it calls (patch_hrc_i_geom, hrc_i_geom.c:119) reads Verbose from a
        # null parameter file (hrc_i_geom.c:190) and fails.  The fixture keeps
        # the inputs and the reference's facet geometry only.
        out["marx2fits"] = np.array("fails: DetectorType HRC-I not supported")
        modes = ()
    else:
        modes = PIXADJ_MODES
    with tempfile.TemporaryDirectory() as tmp:
        for mode in modes:
            c = run_marx2fits(case, ev, U, mode, tmp)
            for col in ("EXPNO", "CHIPX", "CHIPY", "TDETX", "TDETY", "DETX", "DETY", "X", "Y", "FLTGRADE", "GRADE"):
                if col in c:
                    out[f"{mode}_{col.lower()}"] = np.asarray(c[col])
    out["params"] = np.array([case["focal"], *case["det_offset"], case["roll_nom"], FRAME_TIME,
                              float(case["dithered"])])
    out["detector"] = np.array(case["detector"])
    np.savez_compressed(os.path.join(HERE, f"events_{name}.npz"), **out)
    print(name, "events", N_EVENTS, "columns", sorted(k for k in out if k.startswith("EXACT_")))


# ------------------------------------------------------------- ACIS FEF --
FEF_FILE = os.path.join(HERE, "acis_fef_synthetic.fits")
# name: (workload, DetIdeal): with DetIdeal = no the reference also applies
# the CALDB QE and the (synthetic) contamination before the FEF
FEF_CASES = {"fef_acis_i": ("plain_scatter", "yes"), "fef_hetg_s": ("plain_hetg", "yes"),
             "qe_acis_i": ("plain_scatter", "no"), "qe_hetg_s": ("plain_hetg", "no")}


def write_bintable(path, extname, columns, keys=(), tables=None):
    """A FITS file with an empty primary HDU and binary tables:
    columns = [(name, 'J' | 'E' | 'D', values (rows, or rows x repeat))];
    `tables` gives several as [(extname, columns, keys)]."""
    def block(cards):
        h = "".join(c.ljust(80)[:80] for c in cards) + "END".ljust(80)
        return h.ljust((len(h) + 2879) // 2880 * 2880).encode("ascii")
    card = lambda k, v: f"{k:<8}= {v:>20}"
    out = block([card("SIMPLE", "T"), card("BITPIX", "8"), card("NAXIS", "0"), card("EXTEND", "T")])
    for ext, cols, kv in (tables or [(extname, columns, keys)]):
        n = len(cols[0][2])
        vals = [np.asarray(v) for _, _, v in cols]
        reps = [1 if v.ndim == 1 else v.shape[1] for v in vals]
        dt = np.dtype([(name, {"J": ">i4", "E": ">f4", "D": ">f8"}[t], (r,)) if r > 1 else
                       (name, {"J": ">i4", "E": ">f4", "D": ">f8"}[t]) for (name, t, _), r in zip(cols, reps)])
        rec = np.zeros(n, dtype=dt)
        for (name, t, _), v in zip(cols, vals):
            rec[name] = v
        cards = [card("XTENSION", "'BINTABLE'"), card("BITPIX", "8"), card("NAXIS", "2"),
                 card("NAXIS1", str(dt.itemsize)), card("NAXIS2", str(n)), card("PCOUNT", "0"), card("GCOUNT", "1"),
                 card("TFIELDS", str(len(cols)))]
        for i, ((name, t, _), r) in enumerate(zip(cols, reps)):
            cards += [card(f"TTYPE{i + 1}", f"'{name}'"), card(f"TFORM{i + 1}", f"'{r}{t}'")]
        cards += [card("EXTNAME", f"'{ext}'")] + [card(k, v) for k, v in kv]
        data = rec.tobytes()
        data += b"\0" * ((-len(data)) % 2880)
        out += block(cards) + data
    with open(path, "wb") as f:
        f.write(out)


CONTAM_FILE = os.path.join(HERE, "acis_contam_synthetic.fits")


def synthetic_contam():
    """Per chip two layers (component 0), 35 of 40 energy slots and 5 of 6
    time slots used; the spatial term by the reference's own functions,
    except on the BI chips 5 and 7, which carry an fxy map of 32 x 32
    blocks (fxyblk = 32)."""
    tables = []
    e = np.zeros(40, np.float32)
    e[:35] = np.geomspace(0.1, 12.0, 35)
    t = np.zeros(6)
    t[:5] = [-2.0e8, 0.5e8, 1.5e8, 3.0e8, 5.0e8]
    for ccd in range(10):
        mu = np.zeros((2, 40), np.float32)
        mu[0, :35] = 2.2 * e[:35] ** -2.4          # carbon-like
        mu[1, :35] = 0.9 * e[:35] ** -2.0 + 0.05   # a second layer
        tau0 = np.zeros((2, 6), np.float32)
        tau1 = np.zeros((2, 6), np.float32)
        tau0[0, :5] = [0.02, 0.05, 0.08, 0.12, 0.16]
        tau0[1, :5] = [0.01, 0.02, 0.03, 0.04, 0.05]
        tau1[0, :5] = [0.01, 0.03, 0.05, 0.07, 0.09]
        tau1[1, :5] = [0.0, 0.005, 0.01, 0.015, 0.02]
        cols = [("component", "J", np.zeros(2)), ("n_energy", "J", np.full(2, 35)), ("energy", "E", np.tile(e, (2, 1))),
                ("mu", "E", mu), ("n_time", "J", np.full(2, 5)), ("time", "D", np.tile(t, (2, 1))),
                ("tau0", "E", tau0), ("tau1", "E", tau1)]
        keys = ()
        if ccd in (5, 7):
            yy, xx = np.mgrid[0:32, 0:32]
            fxy = (((xx - 15.5) ** 2 + (yy - 15.5) ** 2) / 400.0).astype(np.float32).ravel()
            cols.append(("fxy", "E", np.tile(fxy, (2, 1)) * np.array([[1.0], [0.5]], np.float32)))
            keys = (("FXYBLK", "32"),)
        tables.append((f"ACIS{ccd}_CONTAM", cols, keys))
    return tables


def synthetic_fef():
    """Rows of the synthetic FEF (see the module docstring)."""
    energies = np.geomspace(0.15, 12.0, 20)
    cols = {k: [] for k in ("CCD_ID", "CHIPX_LO", "CHIPX_HI", "CHIPY_LO", "CHIPY_HI", "REGNUM", "ENERGY", "CHANNEL",
                            "G1_FWHM", "G1_POS", "G1_AMPL", "G2_FWHM", "G2_POS", "G2_AMPL",
                            "G3_FWHM", "G3_POS", "G3_AMPL")}
    reg = 0
    for ccd in range(10):
        for rx in range(2):
            for ry in range(2):
                gain = 1.0 + 0.01 * (2 * rx + ry - 1.5) + 0.004 * ccd
                for e in energies:
                    ch = e * 1000.0 / 14.6 * gain
                    fwhm = (55.0 + 45.0 * np.sqrt(e)) / 14.6
                    vals = dict(CCD_ID=ccd, CHIPX_LO=1 + 512 * rx, CHIPX_HI=512 * (rx + 1), CHIPY_LO=1 + 512 * ry,
                                CHIPY_HI=512 * (ry + 1), REGNUM=reg, ENERGY=e, CHANNEL=ch,
                                G1_FWHM=fwhm, G1_POS=ch, G1_AMPL=1.0,
                                G2_FWHM=2.5 * fwhm, G2_POS=0.7 * ch,
                                G2_AMPL=-0.004 if ccd in (5, 7) else 0.04,
                                G3_FWHM=6.0, G3_POS=-5.0, G3_AMPL=0.8 + 0.2 * e)
                    for k, v in vals.items():
                        cols[k].append(v)
                reg += 1
    kinds = {k: ("J" if k in ("CCD_ID", "CHIPX_LO", "CHIPX_HI", "CHIPY_LO", "CHIPY_HI", "REGNUM") else "E")
             for k in cols}
    return [(k, kinds[k], np.array(v)) for k, v in cols.items()]


def fef_datadir(where: str) -> str:
    """A copy of the MARX data directory with the synthetic FEF as its
    caldb/acisfef.fits (the ACISFEF entry of marxcaldb.par)."""
    src = os.path.join(REF_ROOT, "marx", "data")
    dst = os.path.join(where, "data")
    shutil.copytree(src, dst)
    shutil.copy(FEF_FILE, os.path.join(dst, "caldb", "acisfef.fits"))
    shutil.copy(CONTAM_FILE, os.path.join(dst, "caldb", "acisD1999-08-13contamN0015_marx.fits"))
    return dst


def fef_fixtures():
    write_bintable(FEF_FILE, "FUNCTION", synthetic_fef())
    write_bintable(CONTAM_FILE, None, None, tables=synthetic_contam())
    tmp = tempfile.mkdtemp()
    try:
        dd = fef_datadir(tmp)
        for name, (base, ideal) in FEF_CASES.items():
            w = W.ALL[base](parity=True)
            ph = w.photons(N_TRACE, seed=w.seed + 11)
            U, N = predraw_variates(N_TRACE, seed=w.seed + 12)
            ref = Reference(w.cfg, datadir=dd, extra_par={"DetIdeal": ideal})
            q, used, bad = ref.trace_slots(ph, U, N)
            assert bad == 0, "reference ran past its variate slots"
            np.savez_compressed(
                os.path.join(HERE, f"trace_{name}.npz"),
                energy=ph.energy, p_in=ph.p, arrival_time=ph.arrival_time, U=U, N=N,
                x=q.x, p=q.p, flags=q.flags, mirror_shell=q.mirror_shell, order=q.order, ccd_num=q.ccd_num,
                y_pixel=q.y_pixel, z_pixel=q.z_pixel, dither_state=q.dither_state, used=used,
                pulse_height=q.pulse_height, pi=q.pi)
            on_chip = q.ccd_num >= 0
            print(name, "on chips", int(on_chip.sum()), "FEF-detected", int(((q.flags & 0xFF) == 0).sum()),
                  "pha range", q.pulse_height[on_chip].min() if on_chip.any() else None,
                  q.pulse_height[on_chip].max() if on_chip.any() else None)
            ref_n = Reference(w.cfg, native=True, seed=w.seed, datadir=dd, extra_par={"DetIdeal": ideal})
            ph = w.photons(N_STATS, seed=w.seed + 13)
            q, secs = ref_n.trace_batch(ph)
            good = (q.flags & 0xFF) == 0
            hit = q.ccd_num >= 0
            out = {"n": np.array(q.n), "on_chip": np.array(hit.sum()), "good": np.array(good.sum()),
                   "streaked": np.array(((q.flags & 0x200) != 0).sum()),
                   "pha_hist": np.bincount(np.clip(q.pulse_height[good].astype(int), 0, 1023) // 8, minlength=128),
                   "pi_hist": np.histogram(q.pi[good], bins=np.linspace(0, 12, 97))[0]}
            np.savez_compressed(os.path.join(HERE, f"stats_{name}.npz"), **out)
            print(name, "stats", {k: int(v) for k, v in out.items() if v.ndim == 0})
    finally:
        shutil.rmtree(tmp)


ASPSOL_FILE = os.path.join(HERE, "aspsol_synthetic.fits")
ASPSOL_CASES = {"aspsol_scatter": "plain_scatter", "aspsol_hrci": "plain_hrci"}
ASPSOL_KEYS = (("RA_NOM", "83.8221"), ("DEC_NOM", "-5.3911"), ("ROLL_NOM", "250.37"), ("TSTART", "300000000.5"))
ASPSOL_SPAN = 200.0   # s of photon arrival times covered by the table


def synthetic_aspsol():
    """An aspect solution at 0.256 s steps from TSTART - 1 s to TSTART +
    ASPSOL_SPAN + 2 s: Lissajous pointing (8 arcsec, periods 707 and 1000 s)
    about the nominal pointing with a slow roll wobble, and a detector
    drifting by tens of microns and turning by a few arcsec."""
    kv = {k: float(v) for k, v in ASPSOL_KEYS}
    t = kv["TSTART"] - 1.0 + 0.256 * np.arange(int((ASPSOL_SPAN + 3.0) / 0.256))
    s = t - kv["TSTART"]
    a = 8.0 / 3600.0
    ra = kv["RA_NOM"] + a * np.sin(2 * np.pi * s / 707.0) / np.cos(np.radians(kv["DEC_NOM"]))
    dec = kv["DEC_NOM"] + a * np.sin(2 * np.pi * s / 1000.0 + 0.3)
    roll = kv["ROLL_NOM"] + (10.0 / 3600.0) * np.sin(2 * np.pi * s / 150.0)
    dy = 0.02 * np.sin(2 * np.pi * s / 90.0)
    dz = -0.015 * np.cos(2 * np.pi * s / 130.0)
    dth = (4.0 / 3600.0) * np.sin(2 * np.pi * s / 60.0)
    cols = [("time", "D", t), ("ra", "D", ra), ("dec", "D", dec), ("roll", "D", roll), ("dy", "D", dy),
            ("dz", "D", dz), ("dtheta", "D", dth)]
    return cols, list(ASPSOL_KEYS)


def aspsol_fixture(name):
    """trace_<name>.npz: the workload's photons at arrival times spread over
    the aspect solution, traced by the reference with DitherModel = FILE;
    the dither state (sky and detector parts) is recorded with the rest."""
    from marx_gb300.aspsol import read_aspsol, apply_to_config
    cols, keys = synthetic_aspsol()
    write_bintable(ASPSOL_FILE, "ASPSOL", cols, keys)
    asp = read_aspsol(ASPSOL_FILE)
    w = W.ALL[ASPSOL_CASES[name]](parity=True)
    cfg = apply_to_config(w.cfg, asp)
    ph = w.photons(N_TRACE, seed=w.seed + 21)
    ph.arrival_time[:] = np.sort(np.random.default_rng(w.seed + 22).uniform(0.0, ASPSOL_SPAN, N_TRACE))
    U, N = predraw_variates(N_TRACE, seed=w.seed + 23)
    ref = Reference(cfg, extra_par={"DitherModel": "FILE", "DitherFile": ASPSOL_FILE})
    q, used, bad = ref.trace_slots(ph, U, N)
    assert bad == 0, "reference ran past its variate slots"
    assert (used[:, 1] >= 0).all(), "a photon fell outside the aspect solution"
    np.savez_compressed(
        os.path.join(HERE, f"trace_{name}.npz"),
        energy=ph.energy, p_in=ph.p, arrival_time=ph.arrival_time, U=U, N=N,
        x=q.x, p=q.p, flags=q.flags, mirror_shell=q.mirror_shell, order=q.order, ccd_num=q.ccd_num,
        y_pixel=q.y_pixel, z_pixel=q.z_pixel, dither_state=q.dither_state, det_dither=q.det_dither, used=used)
    print(name, "detected", int(((q.flags & 0xFF) == 0).sum()), "det dither range",
          np.abs(q.det_dither).max(axis=1))


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


SAOSAC_ROWS = 3000


def saosac_fixture():
    """Synthetic SAOSAC ray files and the reference's SAOSAC source
    (s-saosac.c) reading them: rays start 0-2 mm in front of the cap plane
    of the file's frame on the four shells' exit annuli, head for the focus
    with a few arcsec of scatter, energies 0.3-8 keV, weights 0.05-1;
    RT_TIME increasing from 5e3 s with two rows earlier than the first
    (dropped by the reader)."""
    r = np.random.default_rng(77)
    n = SAOSAC_ROWS
    radius = r.choice([316.97, 426.35, 482.86, 599.45], n) + r.normal(0.0, 1.5, n)
    phi = r.uniform(0, 2 * np.pi, n)
    y, z = radius * np.cos(phi), radius * np.sin(phi)
    # the file's x = 0 plane is the cap's (the reader places rays there);
    # rays 0-2 mm in front of it head for the focus at MARX's origin
    x = r.uniform(0.0, 2.0, n)
    cap = W.plain_hetg(parity=True).cfg.hrma_cap_x - 0.016750
    d = np.stack([-(cap + x), -y, -z]) + r.normal(0.0, 0.05, (3, n))
    k = d / np.linalg.norm(d, axis=0)
    y0, z0 = y, z
    t = 5000.0 + np.cumsum(r.exponential(0.2, n))
    t[[700, 1900]] = 4000.0          # earlier than the first row: dropped
    e = r.uniform(0.3, 8.0, n)
    w = r.uniform(0.05, 1.0, n)
    cols = [("RT_X", "D", x), ("RT_Y", "D", y0), ("RT_Z", "D", z0), ("RT_COSX", "D", k[0]), ("RT_COSY", "D", k[1]),
            ("RT_COSZ", "D", k[2]), ("RT_KEV", "E", e), ("RT_WGHT", "E", w)]
    files = {"saosac_synthetic.fits": cols + [("RT_TIME", "D", t)], "saosac_notime.fits": cols}
    U = r.random(n)
    out = {"U": U}
    for fname, c in files.items():
        path = os.path.join(HERE, fname)
        write_bintable(path, "RAYTRACE", c)
        cfg = W.plain_hetg(parity=True).cfg
        ref = Reference(cfg, extra_par={"SourceType": "SAOSAC", "SAOSACFile": path, "DitherModel": "INTERNAL"})
        ref.source_open()
        tag = fname.split("_")[1].split(".")[0]
        used = 0
        for b, m in enumerate((1000, 1000, 1500)):
            q = ref.source_batch(m, U[used:])
            for col in ("energy", "x", "p", "arrival_time", "flags", "mirror_shell"):
                out[f"{tag}_{b}_{col}"] = getattr(q, col)
            out[f"{tag}_{b}_n"] = np.array(q.n)
            out[f"{tag}_{b}_rows"] = np.array(q.uniforms_used)   # one uniform per row read
            used += q.uniforms_used
        print(fname, [int(out[f"{tag}_{b}_n"]) for b in range(3)])
    np.savez_compressed(os.path.join(HERE, "saosac.npz"), **out)


N_FD = 200_000
FD_STEP = 2e-3


def diff_fd_fixture():
    """Central differences of the reference's own mirror stage (ideal
    mirror) for the 18 parameters, with common random numbers: every
    perturbed run traces the same rays (the Philox variates of tags
    0 .. N_FD - 1, served as pre-drawn slots), so the differences carry no
    sampling noise; decisions (which shell, hit or miss of a mirror end or
    a strut) are the reference's own at every step."""
    w = diff_workload(n_rays=N_FD)
    cfg = diff_mirror_config(ideal=True)
    cfg.use_blur = 0
    cfg.use_wfold = 0
    o = Oracle(cfg)
    U, N = o.philox_slots(w.cfg.seed, N_FD)
    tags = np.arange(N_FD, dtype=np.uint32)

    def rays(theta):
        tmp = tempfile.mkdtemp(prefix="mxfd")
        try:
            ref = Reference(cfg, datadir=perturbed_datadir(theta, tmp))
            p0 = source_direction(w.cfg.src_y + theta[16], w.cfg.src_z + theta[17])
            ph = PhotonList.from_inputs(np.full(N_FD, w.cfg.energy), np.repeat(p0[:, None], N_FD, 1),
                                        np.zeros(N_FD))
            ph.tag[:] = tags
            q, used, bad = ref.trace_slots(ph, U, N, stages=2)
            assert bad == 0
        finally:
            shutil.rmtree(tmp)
        hit = (q.flags & 0xFF) == 0
        t = -q.x[0] / q.p[0]
        return np.stack([np.where(hit, q.x[1] + t * q.p[1], np.nan), np.where(hit, q.x[2] + t * q.p[2], np.nan),
                         hit.astype(np.float64)])

    dc = w.cfg.copy()
    r0 = rays(np.zeros(NPARAM))
    h0 = r0[2] > 0
    dc.center_y, dc.center_z = float(r0[0][h0].mean()), float(r0[1][h0].mean())
    # the target: the oracle's image at theta_true from rays of another seed
    tc = dc.copy()
    tc.seed = w.target_seed
    _, target = o.weighted(tc, w.theta_true, rays=False)
    out = {"n": np.array(N_FD), "seed": np.array(w.cfg.seed), "h": np.array(FD_STEP),
           "center": np.array([dc.center_y, dc.center_z]), "target": target}
    points = {"true": w.theta_true, "random": np.random.default_rng(7).normal(0.0, 1.0, NPARAM)}
    for name, theta in points.items():
        loss = lambda r: float(np.mean((o.splat(dc, r) - target) ** 2))  # noqa: E731
        r = rays(theta)
        L = np.zeros((NPARAM, 2))
        changed = np.zeros(NPARAM, np.int64)
        for k in range(NPARAM):
            rr = []
            for j, sgn in enumerate((-1.0, 1.0)):
                t = theta.copy()
                t[k] += sgn * FD_STEP
                rr.append(rays(t))
                L[k, j] = loss(rr[-1])
            changed[k] = int(np.sum((rr[0][2] > 0) != (rr[1][2] > 0)))
        out[f"{name}_theta"] = theta
        out[f"{name}_loss"] = np.array(loss(r))
        out[f"{name}_losses"] = L
        out[f"{name}_grad"] = (L[:, 1] - L[:, 0]) / (2.0 * FD_STEP)
        out[f"{name}_changed"] = changed
        print(name, "rays that hit on one side of a step and not the other:", changed.tolist())
    np.savez_compressed(os.path.join(HERE, "diff_fd_reference.npz"), **out)


N_DISPERSED = 1_000_000
DISPERSED_WORKLOADS = ("plain_hetg", "plain_letg", "letg_hrcs")


def dispersed_fixture(name):
    """Dispersed spectra of the reference's seeded run (its own generator):
    per grating arm and order, the detected photons' coordinate along the
    dispersion direction (tests/helpers.py dispersed_groups)."""
    sys.path.insert(0, os.path.dirname(HERE))
    from helpers import dispersed_groups, DISPERSED_BINS
    w = W.ALL[name](parity=True)
    ref_n = Reference(w.cfg, native=True, seed=w.seed + 17)
    ph = w.photons(N_DISPERSED, seed=w.seed + 19)
    q, secs = ref_n.trace_batch(ph)
    out = {"n": np.array(N_DISPERSED)}
    for key, u in dispersed_groups(q, w.cfg).items():
        u = np.sort(u)
        out[f"count_{key}"] = np.array(u.size)
        # histogram over equal-probability bins of the reference's sample
        edges = np.quantile(u, np.linspace(0.0, 1.0, DISPERSED_BINS + 1)) if u.size >= 10 * DISPERSED_BINS else None
        if edges is not None:
            edges[0], edges[-1] = -np.inf, np.inf
            out[f"edges_{key}"] = edges
            out[f"hist_{key}"] = np.histogram(u, edges)[0]
        out[f"sample_{key}"] = u[:: max(1, u.size // 20000)]
    np.savez_compressed(os.path.join(HERE, f"dispersed_{name}.npz"), **out)
    print(name, {k: int(v) for k, v in out.items() if k.startswith("count_")}, f"{secs:.1f} s")


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(HERE))
    names = [a for a in sys.argv[1:] if not a.startswith("-")]
    if "--saosac" in sys.argv:
        saosac_fixture()
    elif "--diff-fd" in sys.argv:
        diff_fd_fixture()
    elif "--dispersed" in sys.argv:
        for n in names or DISPERSED_WORKLOADS:
            dispersed_fixture(n)
    elif "--diff" in sys.argv:
        diff_rays()
    elif "--fef" in sys.argv:
        fef_fixtures()
    elif "--aspsol" in sys.argv:
        if names:
            aspsol_fixture(names[0])
        else:
            import subprocess
            for n in ASPSOL_CASES:
                subprocess.run([sys.executable, __file__, "--aspsol", n], check=True)
    elif "--events" in sys.argv:
        if names:
            events_fixture(names[0])
        else:
            import subprocess
            for n in EVENT_CASES:
                subprocess.run([sys.executable, __file__, "--events", n], check=True)
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
