"""Throughput of the fused photon trace on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl reference]

A step is one pass of the hot path (aspect dither -> HRMA mirror -> grating
-> ACIS detector) over one batch of synthetic photons of the named workload
(default plain_scatter: 1e7 photons, 0.3-8 keV log-uniform, 0-10 arcmin off
axis, 8 arcsec Lissajous dither, mirror blur and WFold scattering, ACIS-I).

value     photons/s with the batch resident in HBM (inputs > L2, so no flush);
          each step restores the batch's input directions and flags, then
          traces it (from 65536 photons: the four wavefront kernels).
e2e       the same metric through mx_trace_host: pinned host buffers in,
          host buffers out, copies inside the timed region.
roofline  the trace kernel against the measured FP64 FMA peak (it is FP64
          bound); algorithmic FP64 operations per photon come from the
          oracle's counting arithmetic on a sample of the same batch.
cpu_baseline  the CPU oracle (a restatement of the reference) on a bounded
          sample, all host threads.
configs   the on-axis (plain_onaxis, 1e6 photons) and HETG (plain_hetg,
          2e7 photons) configurations at their full sizes, each with its own
          value, roofline, e2e and cpu_baseline.
batched   the 256-source workload: one persistent cooperative launch in a
          CUDA graph against 256 sequential plain traces.
differentiable  4e6 weighted rays: gradients/s of forward + MSE + adjoint
          against central finite differences on the same engine, with the
          adjoint's relative error against them.

With --gpus N > 1 (torchrun, one rank per GPU) every rank traces its own
batch (no collective on the data path) and value = all photons / max time.
"""
from __future__ import annotations

import argparse
import contextlib
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "photons/s HRMA+grating+ACIS trace"
# DRAM bytes the four wavefront kernels move per photon of plain_scatter
# (dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture of 2e6
# photons); the traffic of a step grows with its photon count.
TRAFFIC_BYTES_PER_PHOTON = 557.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="plain_scatter")
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--n", type=int, default=0, help="photons per step (default: the workload's size)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the 256-source batched comparison")
    ap.add_argument("--no-diff", action="store_true", help="skip the differentiable-form gradient comparison")
    ap.add_argument("--no-workloads", action="store_true", help="skip the per-workload throughput table")
    ap.add_argument("--no-events", action="store_true", help="skip the marx2fits event-coordinate pass")
    ap.add_argument("--no-configs", action="store_true", help="skip the full-size on-axis and HETG configurations")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index, self.proc, self.lines = index, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0])); mx = float(f[1])
            except ValueError:
                continue
            for k, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(k)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_init(gpus):
    import torch
    rank, world = int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, world):
    from marx_gb300.replicas import max_over_ranks as mor
    return mor(v, world, "cuda")


def cpu_sample(w, n, threads):
    """Oracle throughput (photons/s) on n photons of the workload."""
    from oracle.bindings import Oracle
    o = Oracle(w.cfg)
    ph = w.photons(n, seed=w.seed + 7)
    o.trace(ph.copy(), seed=1, threads=threads)          # warm
    t0 = time.perf_counter()
    o.trace(ph, seed=2, threads=threads)
    return n / (time.perf_counter() - t0)


def batched_flops(sources, n_sample=20_000):
    """Algorithmic FP64 operations of the batch: the oracle's counting
    arithmetic on a sample of each (grating, detector) pair's photons, drawn
    from its sources in proportion to their counts (energies uniform over
    each source's band, each source's direction), times the pair's photons."""
    import numpy as np
    from marx_gb300 import batched as B
    from marx_gb300.photons import PhotonList
    from oracle.bindings import Oracle
    counts = np.array([s.num_photons for s in sources], dtype=np.float64)
    total = counts.sum()
    r = np.random.default_rng(12)
    flops = 0.0
    for g in sorted({s.grating for s in sources}):
        for d in sorted({s.detector for s in sources}):
            idx = [k for k, s in enumerate(sources) if s.grating == g and s.detector == d]
            if not idx:
                continue
            take = [max(1, int(round(n_sample * counts[k] / total))) for k in idx]
            E = np.concatenate([r.uniform(sources[k].energy_min, sources[k].energy_max, m) for k, m in zip(idx, take)])
            P = np.concatenate([np.repeat(np.array(sources[k].p[:])[:, None], m, 1) for k, m in zip(idx, take)], 1)
            cfg = B.batched_config()
            cfg.grating, cfg.detector = g, d
            ops, cnt = Oracle(cfg).count_flops(PhotonList.from_inputs(E, P), seed=5)
            flops += ops / cnt * counts[idx].sum()
    return flops


def bench_batched(a, fp64_peak):
    """256 uneven point sources: one persistent graph launch (after the
    autotuner chose its launch shape) against 256 sequential plain traces
    of the same photons.  Both write identical per-photon results."""
    import torch
    from marx_gb300 import batched as B
    from marx_gb300._native import Engine
    eng = Engine(B.batched_config())
    sources = B.batched_sources()
    b = B.Batch(eng, sources)
    t0 = time.perf_counter()
    params = b.tune(trials=2)
    tune_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()

    def timed(fn, k):
        for s in range(2):
            fn(seed=900 + s)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for s in range(k):
            fn(seed=s)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    k = max(2, min(a.steps, 5))
    ms_b = timed(b.run, k)
    ms_s = timed(b.run_sequential, k)
    flops = batched_flops(sources)
    achieved = flops / (ms_b * 1e-3) / 1e12
    roof = {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s", "frac": achieved / fp64_peak,
            "algorithmic_flops_per_photon": flops / b.n,
            "sequential_frac": flops / (ms_s * 1e-3) / 1e12 / fp64_peak,
            "note": "graph launch time (generation and trace of every source); per-photon operations from the "
                    "oracle's counting arithmetic per (grating, detector) pair"}
    return {"workload": "256 point sources, photons log-uniform 1e3-1e6 per source, 0-10 arcmin, 0.3-10 keV, "
                        "grating NONE|HETG and ACIS-I|ACIS-S per source",
            "photons_per_step": b.n, "steps": k,
            "batched_photons_per_s": b.n / (ms_b * 1e-3), "sequential_photons_per_s": b.n / (ms_s * 1e-3),
            "batched_ms": ms_b, "sequential_ms": ms_s, "speedup": ms_s / ms_b,
            "tuned_params": params, "tune_seconds": tune_s,
            "roofline": roof}


def bench_diff(a, fp64_peak):
    """Differentiable form, 4e6 weighted rays at 1.49 keV, 2' off-axis,
    256 x 256 image, target at the seeded perturbation.  A gradient step is
    forward image (decisions recorded) + MSE + adjoint, all on the device;
    the comparison is the central-difference gradient on the same engine:
    36 forward images (decisions replayed) + 36 MSEs."""
    import numpy as np
    import torch
    from marx_gb300 import diff as D
    from marx_gb300._native import Engine
    from oracle.bindings import Oracle
    eng = Engine(D.diff_mirror_config())
    w = D.diff_workload()
    d = D.DiffImage.centred(eng, w.cfg)
    tc = d.cfg.copy()
    tc.seed = w.target_seed
    dt = D.DiffImage(eng, tc)
    target = dt.forward(w.theta_true, D.FRESH).clone()
    dt.close()
    theta = np.zeros(D.NPARAM)
    stream = torch.cuda.current_stream()
    img = d.new_image()
    grad = torch.zeros(D.NPARAM, dtype=torch.float64, device="cuda")
    loss = torch.zeros((), dtype=torch.float64, device="cuda")
    dl = torch.empty_like(img)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def gradient_step(record_times=False):
        e = [ev() for _ in range(4)] if record_times else None
        if e: e[0].record(stream)
        d.forward(theta, D.RECORD, out=img)
        if e: e[1].record(stream)
        d.L.mx_diff_mse(d.h, img.data_ptr(), target.data_ptr(), dl.data_ptr(), loss.data_ptr(), stream.cuda_stream)
        if e: e[2].record(stream)
        d.adjoint_async(theta, dl, grad)
        if e:
            e[3].record(stream)
            return e
        return None

    for _ in range(max(a.warmup, 3)):
        gradient_step()
    torch.cuda.synchronize()
    k = max(3, a.steps)
    marks = []
    launches0 = eng.launch_count()
    t0, t1 = ev(), ev()
    t0.record(stream)
    for _ in range(k):
        marks.append(gradient_step(True))
    t1.record(stream)
    torch.cuda.synchronize()
    launches = eng.launch_count() - launches0
    grad_ms = t0.elapsed_time(t1) / k
    fwd_ms = statistics.mean(m[0].elapsed_time(m[1]) for m in marks)
    adj_ms = statistics.mean(m[2].elapsed_time(m[3]) for m in marks)
    g_adj = grad.cpu().numpy()
    fd_gradient = D.fd_gradient
    fd_gradient(d, theta, target)                      # warm
    torch.cuda.synchronize()
    kf = 2
    t0.record(stream)
    for _ in range(kf):
        g_fd = fd_gradient(d, theta, target)
    t1.record(stream)
    torch.cuda.synchronize()
    fd_ms = t0.elapsed_time(t1) / kf
    rel = np.abs(g_adj - g_fd) / np.abs(g_fd)
    # end to end through the host entry points: theta in, loss and gradient
    # back to host memory every step (mx_diff_adjoint waits for the stream)
    for _ in range(2):
        d.forward(theta, D.RECORD, out=img)
        d.mse(img, target, loss=loss)
        d.adjoint(theta, dl)
    torch.cuda.synchronize()
    with no_gc():
        h0 = time.perf_counter()
        for _ in range(k):
            d.forward(theta, D.RECORD, out=img)
            d.L.mx_diff_mse(d.h, img.data_ptr(), target.data_ptr(), dl.data_ptr(), loss.data_ptr(), stream.cuda_stream)
            g_host = d.adjoint(theta, dl)
            _ = float(loss.item())
        e2e_s = (time.perf_counter() - h0) / k
    ops = Oracle(D.diff_mirror_config()).weighted_flops(D.diff_workload(n_rays=20000).cfg, theta)
    flops_per_ray = ops[0] / ops[1]
    n = w.cfg.n_rays
    fwd_tf = flops_per_ray * n / (fwd_ms * 1e-3) / 1e12
    adj_tf = flops_per_ray * n / (adj_ms * 1e-3) / 1e12
    return {"workload": "4e6 weighted rays, 1.49 keV, 2 arcmin off-axis, 256x256 image of 24 um pixels, "
                        "Gaussian sigma 1 pixel, MSE to a target at per-shell tilts N(0,2\"), decenters "
                        "N(0,10 um), source offset N(0,0.5\")",
            "rays": n, "parameters": D.NPARAM, "steps": k,
            "gradients_per_s": 1e3 / grad_ms, "gradient_ms": grad_ms,
            "fd_gradients_per_s": 1e3 / fd_ms, "fd_gradient_ms": fd_ms, "speedup_vs_fd": fd_ms / grad_ms,
            "forward_ms": fwd_ms, "adjoint_ms": adj_ms,
            "max_rel_err_vs_fd": float(rel.max()), "norm_rel_err_vs_fd": float(np.linalg.norm(g_adj - g_fd) /
                                                                              np.linalg.norm(g_fd)),
            "fd_step": 2e-3, "gpu_launches": launches,
            "e2e": {"gradients_per_s": 1.0 / e2e_s, "h2d_bytes_per_step": 2 * 8 * D.NPARAM,
                    "d2h_bytes_per_step": 8 * (D.NPARAM + 1),
                    "note": "theta from the host into the forward and adjoint calls, loss and gradient read back "
                            "to host each step; target image resident"},
            "roofline": {"bound": "fp64", "unit": "TFLOP/s", "peak": fp64_peak,
                         "algorithmic_flops_per_ray": flops_per_ray,
                         "forward": {"achieved": fwd_tf, "frac": fwd_tf / fp64_peak},
                         "adjoint": {"achieved": adj_tf, "frac": adj_tf / fp64_peak,
                                     "note": "FP64 values only; the six FP32 tangents per value are not counted"}},
            }


def bench_workloads(a, skip):
    """Photons/s of every other named workload (device-resident batch, the
    kernels alone): the plain configurations, the LETG and the HRC."""
    import torch
    from marx_gb300 import workloads as W
    from marx_gb300._native import Engine, DevicePhotons
    out = {}
    stream = torch.cuda.current_stream()
    for name, make in W.ALL.items():
        if name in skip:
            continue
        w = make()
        n = min(w.n, 4_000_000)
        eng = Engine(w.cfg)
        d = DevicePhotons.from_host(w.photons(n, seed=w.seed + 5))
        p0, f0 = d.p.clone(), d.flags.clone()
        for s in range(2):
            d.p.copy_(p0); d.flags.copy_(f0)
            eng.trace(d, stages=w.stages, seed=700 + s)
        torch.cuda.synchronize()
        k = max(3, min(a.steps, 5))
        ms = 0.0
        for s in range(k):
            d.p.copy_(p0); d.flags.copy_(f0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.trace(d, stages=w.stages, seed=s)
            e1.record(stream)
            torch.cuda.synchronize()
            ms += e0.elapsed_time(e1)
        ms /= k
        good = float(((d.flags & 0xFF) == 0).float().mean().item())
        out[name] = {"photons": n, "ms": ms, "photons_per_s": n / (ms * 1e-3), "detected_fraction": good}
        eng.close()
        del d
    out.update(bench_fef(a))
    return out


def bench_fef(a):
    """plain_scatter with an ACIS FEF in the tables (the synthetic FEF the
    tests pin against the reference): the trace plus the FEF pass."""
    import tempfile
    import torch
    from marx_gb300 import workloads as W
    from marx_gb300._native import Engine, DevicePhotons
    from marx_gb300.caldb.pack import DEFAULT_PACK, pack_with_fef
    fef = os.path.join(ROOT, "tests", "golden", "acis_fef_synthetic.fits")
    if not os.path.exists(fef):
        return {}
    with tempfile.TemporaryDirectory() as tmp:
        pack = os.path.join(tmp, "fef.mxpack")
        pack_with_fef(DEFAULT_PACK, fef, pack)
        w = W.ALL["plain_scatter"]()
        n = 4_000_000
        eng = Engine(w.cfg, pack=pack)
    d = DevicePhotons.from_host(w.photons(n, seed=w.seed + 6))
    p0, f0 = d.p.clone(), d.flags.clone()
    stream = torch.cuda.current_stream()
    for s in range(2):
        d.p.copy_(p0); d.flags.copy_(f0)
        eng.trace(d, stages=w.stages, seed=800 + s)
    torch.cuda.synchronize()
    k = max(3, min(a.steps, 5))
    ms = 0.0
    for s in range(k):
        d.p.copy_(p0); d.flags.copy_(f0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.trace(d, stages=w.stages, seed=s)
        e1.record(stream)
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
    ms /= k
    good = float(((d.flags & 0xFF) == 0).float().mean().item())
    eng.close()
    return {"plain_scatter_fef": {"photons": n, "ms": ms, "photons_per_s": n / (ms * 1e-3), "detected_fraction": good,
                                  "note": "with the synthetic ACIS FEF: trace, then the FEF pulse-height pass"}}


EVENT_BYTES = 1 + 4 + 4 + 4 + 12 + 4 + 4 + 4 + 8 + 8 + 8 + 8 + 4 + 4 + 4 + 2 + 2   # columns read + written


def bench_events(a):
    """The marx2fits event pass (mx_event_coords) on 1e7 ACIS-I events in
    device memory: EDSER sub-pixel positions, INTERNAL dither with frames of
    ~30 events, Philox grade draws; the oracle restatement timed on a sample
    of the same events on one host core."""
    import torch
    from marx_gb300 import workloads as W, events as E
    from marx_gb300._native import Engine
    n = 10_000_000
    g = torch.Generator(device="cuda").manual_seed(31)
    dev = "cuda"
    frame = E.ACIS_FRAME_TIME
    t = torch.sort(torch.rand(n, generator=g, device=dev) * (n / 30 * frame)).values.float()
    arc = 3.141592653589793 / 648000.0
    ev = {"ccd": torch.randint(0, 4, (n,), generator=g, device=dev, dtype=torch.int8),
          "xpixel": torch.rand(n, generator=g, device=dev) * 1024, "ypixel": torch.rand(n, generator=g, device=dev) * 1024,
          "time": t, "sky_ra": (8 * arc * torch.sin(t / 159.0)).float(), "sky_dec": (8 * arc * torch.sin(t / 112.5)).float(),
          "sky_roll": torch.full((n,), 4.137, device=dev), "b_energy": 0.3 + 9.7 * torch.rand(n, generator=g, device=dev)}
    eng = Engine(W.ALL["plain_scatter"]().cfg)
    p = E.params(roll_nom=237.36968458476, dithered=True, pixel_adjust="EDSER")
    stream = torch.cuda.current_stream()
    for s in range(3):
        E.event_coords(eng, p, ev, n, seed=s)
    torch.cuda.synchronize()
    k = max(3, min(a.steps, 10))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = eng.launch_count()
    e0.record(stream)
    for s in range(k):
        E.event_coords(eng, p, ev, n, seed=100 + s)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / k
    launches = (eng.launch_count() - l0) // k
    hbm_peak = 6800.0
    try:
        hbm_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, KeyError, ValueError):
        pass
    gbs = EVENT_BYTES * n / (ms * 1e-3) / 1e9
    # the oracle restatement on a sample of the same events (checker only)
    import numpy as np
    from oracle.event_coords import event_coords as oracle_events, subpix_tables
    from marx_gb300.caldb.pack import DEFAULT_PACK, read_pack
    z = np.load(os.path.join(ROOT, "tests", "golden", "events_acis_i.npz"))
    m = 200_000
    host = {k: v[:m].cpu().numpy() for k, v in ev.items()}
    for c in ("det_dy", "det_dz", "det_theta"):
        host[c] = np.zeros(m, np.float32)
    sub = subpix_tables(read_pack(DEFAULT_PACK))
    prm = dict(focal_length=10070.0, det_offset=(0.0, 0.0, 0.0), roll_nom=237.36968458476, frame_time=frame,
               dithered=True, pixel_adjust=0)
    c0 = time.perf_counter()
    oracle_events("ACIS-I", z["geom"], z["tdet"], z["fp"], prm, host, np.random.default_rng(1).random((3, m)), sub)
    cpu_rate = m / (time.perf_counter() - c0)
    eng.close()
    return {"workload": "1e7 ACIS-I events, EDSER, INTERNAL dither, frames of ~30 events, device-resident",
            "events": n, "ms": ms, "events_per_s": n / (ms * 1e-3), "gpu_launches_per_step": launches,
            "roofline": {"bound": "fp64", "note": "sin, cos, acos, asin, atan and about 26 divisions per event; "
                                                  "ncu: FP64 pipe 87% busy",
                         "hbm": {"achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                                 "bytes_per_event": EVENT_BYTES}},
            "cpu_baseline": {"value": cpu_rate, "unit": "events/s", "cores": 1, "kind": "port",
                             "sample": f"{m} of the same events through the numpy restatement"}}


def run_reference(a):
    """Reference arm: the CPU implementation of the path on the host cores."""
    from marx_gb300 import workloads as W
    rank, world = int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))
    if rank != 0:
        return
    w = W.PLAIN[a.workload]()
    threads = os.cpu_count() or 1
    n = 400_000
    for _ in range(max(a.warmup, 0)):
        cpu_sample(w, 50_000, threads)
    rates = [cpu_sample(w, n, threads) for _ in range(a.steps)]
    v = statistics.median(rates)
    line = {"metric": METRIC, "value": v, "unit": "photons/s", "impl": "reference", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": n / v * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": a.workload, "photons_per_step": n, "sample_of": w.n},
            "cpu_baseline": {"value": v, "unit": "photons/s", "cores": threads, "kind": "port",
                             "sample": f"{n} photons of {a.workload} per step"},
            "e2e": {"value": v, "unit": "photons/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


@contextlib.contextmanager
def no_gc():
    """Python's cyclic garbage collector off around a wall-clock timed loop
    (as timeit does): a collection pause belongs to the harness, not to the
    call being timed."""
    gc.collect()
    was = gc.isenabled()
    gc.disable()
    try:
        yield
    finally:
        if was:
            gc.enable()


def e2e_host(eng, host, w, n, steps, warmup, world=1):
    """The metric through mx_trace_host: pinned host buffers in, every
    output column back in host memory, wall clock around each blocking
    call."""
    import numpy as np
    import torch
    from marx_gb300.photons import PhotonList
    pin = {}
    for k in ("energy", "p", "arrival_time", "flags", "tag", "x", "mirror_shell", "order", "ccd_num",
              "y_pixel", "z_pixel", "dither_state"):
        src = getattr(host, k)
        t = torch.empty(src.shape, dtype=getattr(torch, str(src.dtype).replace("uint32", "int32")), pin_memory=True)
        t.numpy()[...] = src.view(np.int32) if src.dtype == np.uint32 else src
        pin[k] = t
    hp = PhotonList.__new__(PhotonList)
    hp.n = n
    for k, t in pin.items():
        arr = t.numpy()
        setattr(hp, k, arr.view(np.uint32) if k in ("flags", "tag") else arr)
    p_in = pin["p"].clone()
    in_b = sum(pin[k].numel() * pin[k].element_size() for k in ("energy", "p", "arrival_time", "flags", "tag"))
    out_b = sum(pin[k].numel() * pin[k].element_size() for k in ("x", "p", "flags", "mirror_shell", "order",
                                                                 "ccd_num", "y_pixel", "z_pixel", "dither_state"))
    for s in range(max(1, warmup)):
        pin["p"].copy_(p_in); pin["flags"].zero_()
        eng.trace_host(hp, stages=w.stages, seed=2000 + s)
    barrier(world)
    e2e_s = 0.0
    with no_gc():
        for s in range(steps):
            # the step's inputs are put back in the pinned buffers outside the
            # timed region; each timed call copies them in, traces and copies
            # every output column back
            pin["p"].copy_(p_in); pin["flags"].zero_()
            t0 = time.perf_counter()
            eng.trace_host(hp, stages=w.stages, seed=s)
            e2e_s += time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, world)
    barrier(world)
    return {"value": world * n * steps / e2e_s, "unit": "photons/s",
            "h2d_bytes_per_step": in_b, "d2h_bytes_per_step": out_b,
            "note": "pinned host buffers; wall clock around each blocking mx_trace_host call (copies in, "
                    "trace, copies out; the host-side reset of the step's inputs is not timed; Python's "
                    "garbage collector off during the timed steps)"}


def flops_per_photon(w):
    """Algorithmic FP64 operations per photon: the oracle's counting
    arithmetic on 2e4 photons of the workload."""
    from oracle.bindings import Oracle
    sample = w.photons(20_000, seed=w.seed + 99)
    ops, cnt = Oracle(w.cfg).count_flops(sample, seed=5)
    return ops / cnt


def bench_config(a, name, fp64_peak):
    """One configuration at its full size on one GPU: photons/s with the
    batch resident (every launch timed with CUDA events on the launching
    stream), the FP64 roofline of the trace, the same through
    mx_trace_host, and the oracle on a sample."""
    import torch
    from marx_gb300 import workloads as W
    from marx_gb300._native import Engine, DevicePhotons
    w = W.PLAIN[name]()
    n = w.n
    eng = Engine(w.cfg)
    host = w.photons(n)
    d = DevicePhotons.from_host(host)
    p0, f0 = d.p.clone(), d.flags.clone()
    stream = torch.cuda.current_stream()
    for s in range(max(3, a.warmup)):
        d.p.copy_(p0); d.flags.copy_(f0)
        eng.trace(d, stages=w.stages, seed=1000 + s)
    torch.cuda.synchronize()
    k = max(3, min(a.steps, 10))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = eng.launch_count()
    t0.record(stream)
    for s in range(k):
        d.p.copy_(p0); d.flags.copy_(f0)
        ev[s][0].record(stream)
        eng.trace(d, stages=w.stages, seed=s)
        ev[s][1].record(stream)
    t1.record(stream)
    torch.cuda.synchronize()
    launches = (eng.launch_count() - l0) // k
    ms_step = t0.elapsed_time(t1) / k
    kernel_ms = statistics.mean(e0.elapsed_time(e1) for e0, e1 in ev)
    good = float(((d.flags & 0xFF) == 0).float().mean().item())
    del d, p0, f0
    e2e = e2e_host(eng, host, w, n, k, 1)
    fpp = flops_per_photon(w)
    achieved = fpp * n / (kernel_ms * 1e-3) / 1e12
    cpu_n = 200_000
    cpu_rate = cpu_sample(w, cpu_n, os.cpu_count() or 1)
    eng.close()
    torch.cuda.empty_cache()
    return {"workload": name, "photons_per_step": n, "steps": k, "value": n / (ms_step * 1e-3), "unit": "photons/s",
            "ms_per_step": ms_step, "kernel_ms": kernel_ms, "gpu_launches_per_step": launches,
            "detected_fraction": good,
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp64_peak, "traffic": None,
                         "algorithmic_flops_per_photon": fpp,
                         "peak_source": "measured live: mx_probe_fp64 DFMA kernel"},
            "e2e": e2e,
            "cpu_baseline": {"value": cpu_rate, "unit": "photons/s", "cores": os.cpu_count() or 1, "kind": "port",
                             "sample": f"{cpu_n} photons of {name}"}}


def main():
    a = parse()
    if a.impl == "reference":
        return run_reference(a)
    import torch
    from marx_gb300 import workloads as W
    from marx_gb300._native import Engine, DevicePhotons, probe_fp64

    rank, world = dist_init(a.gpus)
    dev = torch.cuda.current_device()
    w = W.PLAIN[a.workload]()
    n = a.n or w.n
    eng = Engine(w.cfg)

    from marx_gb300.replicas import rank_photons
    host = rank_photons(w, n, rank)
    d = DevicePhotons.from_host(host)
    p0, flags0 = d.p.clone(), d.flags.clone()
    stream = torch.cuda.current_stream()

    def step(seed):
        d.p.copy_(p0)
        d.flags.copy_(flags0)
        eng.trace(d, stages=w.stages, seed=seed)

    for s in range(a.warmup):
        step(1000 + s)
    torch.cuda.synchronize()
    # kernel-only timing of the same launches for the roofline
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    launches0 = eng.launch_count()
    with ClockSampler(dev) as clocks:
        barrier(world)
        torch.cuda.synchronize()
        t_start = torch.cuda.Event(enable_timing=True); t_stop = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for s in range(a.steps):
            d.p.copy_(p0)
            d.flags.copy_(flags0)
            ev[s][0].record(stream)
            eng.trace(d, stages=w.stages, seed=s)
            ev[s][1].record(stream)
        t_stop.record(stream)
        torch.cuda.synchronize()
        barrier(world)
    launches = eng.launch_count() - launches0
    ms_total = t_start.elapsed_time(t_stop)
    kernel_ms = statistics.mean(e0.elapsed_time(e1) for e0, e1 in ev)
    ms_total = max_over_ranks(ms_total, world)
    value = world * n * a.steps / (ms_total * 1e-3)
    good = float(((d.flags & 0xFF) == 0).float().mean().item())

    # end to end through the host entry point, pinned buffers
    e2e = None if a.no_e2e else e2e_host(eng, host, w, n, a.steps, a.warmup, world)

    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    # roofline: algorithmic FP64 operations per photon from the oracle's counting arithmetic
    fpp = flops_per_photon(w)
    fp64_peak = probe_fp64()
    achieved = fpp * n / (kernel_ms * 1e-3) / 1e12
    bytes_per_photon = 8 + 24 + 8 + 4 + 4 + 24 + 24 + 4 + 3 + 8 + 12 + 24   # SoA columns read + written
    hbm_peak = None
    try:
        hbm_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, KeyError, ValueError):
        hbm_peak = 6800.0
    hbm_achieved = bytes_per_photon * n / (kernel_ms * 1e-3) / 1e9
    cpu_rate = cpu_sample(w, 200_000, os.cpu_count() or 1)
    del d, p0, flags0
    torch.cuda.empty_cache()
    def section(fn, *args):
        # a failing section is reported in its place; the headline line stands
        try:
            return fn(*args)
        except Exception as e:  # noqa: BLE001
            return {"error": f"{type(e).__name__}: {e}"}

    configs = None if a.no_configs else {c: section(bench_config, a, c, fp64_peak)
                                         for c in ("plain_onaxis", "plain_hetg") if c != a.workload}
    batched = None if a.no_batched else section(bench_batched, a, fp64_peak)
    differentiable = None if a.no_diff else section(bench_diff, a, fp64_peak)
    workloads = None if a.no_workloads else section(
        bench_workloads, a, {a.workload} | (set() if a.no_configs else {"plain_onaxis", "plain_hetg"}))
    events = None if a.no_events else section(bench_events, a)

    line = {
        "metric": METRIC, "value": value, "unit": "photons/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_total / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": a.workload, "photons_per_step": n, "parallelism": f"replicas{world}",
                   "l2": "inputs larger than L2 (no flush)", "variates": "philox4x32-10",
                   "detected_fraction": good},
        "e2e": e2e,
        "gpu_launches": launches,
        "kernel_ms": kernel_ms,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp64_peak,
                     "traffic": TRAFFIC_BYTES_PER_PHOTON * n if a.workload == "plain_scatter" else None,
                     "traffic_note": "bytes per step of the four wavefront kernels, scaled from an ncu capture "
                                     "of 2e6 photons",
                     "algorithmic_flops_per_photon": fpp,
                     "peak_source": "measured live: mx_probe_fp64 DFMA kernel (MEASURED_PEAKS.json has no FP64 figure)",
                     "hbm": {"achieved_gbs": hbm_achieved, "peak_gbs": hbm_peak, "frac": hbm_achieved / hbm_peak,
                             "bytes_per_photon": bytes_per_photon}},
        "cpu_baseline": {"value": cpu_rate, "unit": "photons/s", "cores": os.cpu_count() or 1, "kind": "port",
                         "sample": f"200000 photons of {a.workload}"},
        "clocks": clocks.summary(),
        "configs": configs,
        "batched": batched,
        "differentiable": differentiable,
        "workloads": workloads,
        "events": events,
    }
    print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
