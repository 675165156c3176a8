"""ctypes bindings for the CPU checkers (test infrastructure only)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from marx_gb300.config import MxConfig, to_par
from marx_gb300.photons import MxPhotons, PhotonList, NUM_U, NUM_N

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libmx_oracle.so")
REF_SLOTS_SO = os.path.join(HERE, "_ref", "libmxref_slots.so")
REF_NATIVE_SO = os.path.join(HERE, "_ref", "libmxref_native.so")


def _reference_root() -> str:
    """The reference checkout: MARX_REFERENCE_ROOT, else the one the build
    recipe (oracle/Makefile, REF) names."""
    root = os.environ.get("MARX_REFERENCE_ROOT")
    if root:
        return root
    try:
        r = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "print-ref"], capture_output=True,
                           text=True, timeout=30)
        return r.stdout.strip() if r.returncode == 0 else ""
    except (OSError, subprocess.TimeoutExpired):
        return ""


REF_ROOT = _reference_root()


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_SO


def reference_available() -> bool:
    return bool(REF_ROOT) and os.path.isdir(os.path.join(REF_ROOT, "marx", "libsrc"))


def build_reference() -> bool:
    if not reference_available():
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", "m2f", f"REF={REF_ROOT}"], check=True)
    return True


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(0)


class Oracle:
    """The C++ restatement (oracle/mx_oracle_core.hpp)."""

    def __init__(self, cfg: MxConfig, pack: str | None = None):
        if not os.path.exists(PORT_SO):
            build_port()
        self.lib = C.CDLL(PORT_SO)
        L = self.lib
        L.mxo_create.restype = C.c_void_p
        L.mxo_create.argtypes = [C.c_char_p, C.POINTER(MxConfig)]
        L.mxo_last_error.restype = C.c_char_p
        L.mxo_trace.argtypes = [C.c_void_p, C.POINTER(MxPhotons), C.c_uint32, C.c_void_p, C.c_void_p,
                                C.c_uint64, C.c_int]
        L.mxo_count_flops.argtypes = [C.c_void_p, C.POINTER(MxPhotons), C.c_uint32, C.c_uint64, C.c_void_p]
        L.mxo_detector_geometry.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.mxo_destroy.argtypes = [C.c_void_p]
        L.mxo_philox_uniform.restype = C.c_double
        L.mxo_philox_uniform.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32]
        L.mxo_philox_normal.restype = C.c_double
        L.mxo_philox_normal.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32]
        L.mxo_source_uniform.restype = C.c_double
        L.mxo_source_uniform.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32]
        from marx_gb300.diff import MxDiffConfig
        L.mxo_weighted_flops.argtypes = [C.c_void_p, C.POINTER(MxDiffConfig), C.c_void_p, C.c_void_p]
        L.mxo_splat_exp.restype = C.c_float
        L.mxo_splat_exp.argtypes = [C.c_float]
        L.mxo_weighted.argtypes = [C.c_void_p, C.POINTER(MxDiffConfig), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.mxo_splat.argtypes = [C.POINTER(MxDiffConfig), C.c_void_p, C.c_uint64, C.c_void_p]
        L.mxo_philox_slots.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_void_p, C.c_void_p]
        if pack is None:
            from marx_gb300.caldb.pack import DEFAULT_PACK
            pack = DEFAULT_PACK
        self.cfg = cfg
        self.h = L.mxo_create(pack.encode(), C.byref(cfg))
        if not self.h:
            raise RuntimeError("oracle: " + L.mxo_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.mxo_destroy(self.h)
            self.h = None

    def trace(self, ph: PhotonList, stages: int = 15, U=None, N=None, seed: int = 0, threads: int = 0) -> int:
        s = ph.struct()
        r = self.lib.mxo_trace(self.h, C.byref(s), stages, _p(U), _p(N), seed, threads)
        if r < 0:
            raise RuntimeError(f"oracle trace failed: {r}")
        return r

    def count_flops(self, ph: PhotonList, stages: int = 15, seed: int = 0):
        s = ph.struct()
        out = np.zeros(2)
        self.lib.mxo_count_flops(self.h, C.byref(s), stages, seed, _p(out))
        return out[0], out[1]

    def detector_geometry(self) -> np.ndarray:
        g = np.zeros((10, 20))
        n = self.lib.mxo_detector_geometry(self.h, _p(g), 10)
        return g[:n]

    def philox_uniform(self, seed, tag, slot):
        return self.lib.mxo_philox_uniform(seed, tag, slot)

    def philox_normal(self, seed, tag, slot):
        return self.lib.mxo_philox_normal(seed, tag, slot)

    def source_uniform(self, seed, tag, k=0):
        return self.lib.mxo_source_uniform(seed, tag, k)

    def weighted_flops(self, dcfg, theta):
        """(FP64 operations, rays, rays reaching the focal plane) of the
        weighted rays at theta, from the counting arithmetic."""
        th = np.ascontiguousarray(theta, dtype=np.float64)
        out = np.zeros(3)
        if self.lib.mxo_weighted_flops(self.h, C.byref(dcfg), _p(th), _p(out)) != 0:
            raise RuntimeError("oracle weighted flop count failed")
        return out

    def splat(self, dcfg, yzw):
        """The engine's fixed-point image of given rays (3, n): y, z (mm),
        weight."""
        yzw = np.ascontiguousarray(yzw, dtype=np.float64)
        img = np.zeros((dcfg.ny, dcfg.nx))
        if self.lib.mxo_splat(C.byref(dcfg), _p(yzw), yzw.shape[1], _p(img)) != 0:
            raise RuntimeError("oracle splat failed")
        return img

    def philox_slots(self, seed, n, first_tag=0):
        """Slot arrays (U, N) of the Philox variates of n consecutive tags."""
        U = np.zeros((NUM_U, n))
        N = np.zeros((NUM_N, n))
        self.lib.mxo_philox_slots(seed, first_tag, n, _p(U), _p(N))
        return U, N

    def splat_exp(self, x: float) -> float:
        return self.lib.mxo_splat_exp(x)

    def weighted(self, dcfg, theta, rays: bool = True, image: bool = True, threads: int = 0):
        """Weighted rays of the differentiable form at theta (decisions made
        afresh): (yzw (3, n) or None, image (ny, nx) or None)."""
        th = np.ascontiguousarray(theta, dtype=np.float64)
        yzw = np.zeros((3, dcfg.n_rays)) if rays else None
        img = np.zeros((dcfg.ny, dcfg.nx)) if image else None
        r = self.lib.mxo_weighted(self.h, C.byref(dcfg), _p(th), _p(yzw), _p(img), threads)
        if r != 0:
            raise RuntimeError(f"oracle weighted rays failed: {r}")
        return yzw, img


class Reference:
    """The reference MARX library compiled from its own sources (only in a
    checkout that has them).  ``native=True`` keeps its own generator."""

    def __init__(self, cfg: MxConfig, native: bool = False, seed: int = 1, datadir: str | None = None,
                 extra_par: dict | None = None):
        so = REF_NATIVE_SO if native else REF_SLOTS_SO
        if not os.path.exists(so):
            if not build_reference():
                raise RuntimeError("reference sources not available")
        self.native = native
        self.lib = C.CDLL(so)
        L = self.lib
        L.mxref_last_error.restype = C.c_char_p
        L.mxref_focal_length.restype = C.c_double
        par = to_par(cfg)
        par.update(extra_par or {})
        names = (C.c_char_p * len(par))(*[k.encode() for k in par])
        vals = (C.c_char_p * len(par))(*[v.encode() for v in par.values()])
        parfile = os.path.join(REF_ROOT, "marx", "par", "marx.par").encode()
        datadir = (datadir or os.path.join(REF_ROOT, "marx", "data")).encode()
        if native:
            L.mxref_seed(C.c_ulong(seed))
        r = L.mxref_setup(parfile, datadir, len(par), names, vals)
        if r != 0:
            raise RuntimeError("reference setup: " + L.mxref_last_error().decode())

    def detector_geometry(self) -> np.ndarray:
        g = np.zeros((10, 20))
        n = self.lib.mxref_detector_geometry(_p(g), 10)
        return g[:n]

    def facet_tdet(self) -> np.ndarray:
        t = np.zeros((10, 2))
        n = self.lib.mxref_facet_tdet(_p(t), 10)
        return t[:n]

    def fp_system(self) -> np.ndarray:
        f = np.zeros(3)
        if self.lib.mxref_fp_system(_p(f)) != 0:
            raise RuntimeError("no focal-plane system")
        return f

    def _outs(self, n):
        o = dict(x=np.zeros((n, 3)), p=np.zeros((n, 3)), flags=np.zeros(n, np.uint32),
                 shell=np.zeros(n, np.int32), order=np.zeros(n, np.int32), ccd=np.zeros(n, np.int32),
                 ypix=np.zeros(n, np.float32), zpix=np.zeros(n, np.float32),
                 dith=np.zeros((n, 3), np.float32), sup=np.zeros((n, 4), np.int8), pha=np.zeros(n, np.int16),
                 u=np.zeros(n, np.float32), v=np.zeros(n, np.float32), region=np.zeros(n, np.uint8),
                 pi=np.zeros(n, np.float32), ddith=np.zeros((n, 3), np.float32))
        self.lib.mxref_set_extra_outputs(_p(o["sup"]), _p(o["pha"]), _p(o["u"]), _p(o["v"]), _p(o["region"]))
        self.lib.mxref_set_pi_output(_p(o["pi"]))
        self.lib.mxref_set_det_dither_output(_p(o["ddith"]))
        return o

    def _to_list(self, ph: PhotonList, o: dict) -> PhotonList:
        self.lib.mxref_set_extra_outputs(None, None, None, None, None)
        self.lib.mxref_set_pi_output(None)
        self.lib.mxref_set_det_dither_output(None)
        q = ph.copy()
        q.det_dither = np.ascontiguousarray(o["ddith"].T)
        q.x[:] = o["x"].T; q.p[:] = o["p"].T; q.flags[:] = o["flags"]
        q.mirror_shell[:] = o["shell"]; q.order[:] = o["order"]; q.ccd_num[:] = o["ccd"]
        q.y_pixel[:] = o["ypix"]; q.z_pixel[:] = o["zpix"]; q.dither_state[:] = o["dith"].T
        q.support_orders[:] = o["sup"].T; q.pulse_height[:] = o["pha"]; q.u_pixel[:] = o["u"]
        q.v_pixel[:] = o["v"]; q.detector_region[:] = o["region"]; q.pi[:] = o["pi"]
        return q

    def trace_slots(self, ph: PhotonList, U, N, stages: int = 15):
        """Per-photon run with pre-drawn slot variates (slot-major U, N)."""
        assert not self.native
        n = ph.n
        E = np.ascontiguousarray(ph.energy); P = np.ascontiguousarray(ph.p.T); T = np.ascontiguousarray(ph.arrival_time)
        Up = np.ascontiguousarray(U.T); Np = np.ascontiguousarray(N.T)
        o = self._outs(n)
        used = np.zeros((n, 8), np.int32)
        r = self.lib.mxref_trace_slots(n, _p(E), _p(P), _p(T), _p(Up), _p(Np), stages,
                                       _p(o["x"]), _p(o["p"]), _p(o["flags"]), _p(o["shell"]), _p(o["order"]),
                                       _p(o["ccd"]), _p(o["ypix"]), _p(o["zpix"]), _p(o["dith"]), _p(used))
        if r < 0:
            raise RuntimeError("reference trace: " + self.lib.mxref_last_error().decode())
        return self._to_list(ph, o), used, r

    def dump_rayfile(self, ph: PhotonList, history: int, path: str, new: bool = True, total_time: float = 0.0):
        """The reference's marx_dump_to_rayfile over ph (host columns)."""
        c = lambda a, dt: np.ascontiguousarray(a, dtype=dt)
        f = self.lib.mxref_dump_rayfile
        f.argtypes = [C.c_char_p, C.c_int] + [C.c_void_p] * 18 + [C.c_ulong, C.c_int, C.c_double]
        cols = [c(ph.energy, np.float64), c(ph.x, np.float64), c(ph.p, np.float64), c(ph.arrival_time, np.float64),
                c(ph.flags, np.uint32), c(ph.tag, np.uint32), c(ph.mirror_shell, np.int8), c(ph.order, np.int8),
                c(ph.ccd_num, np.int8), c(ph.y_pixel, np.float32), c(ph.z_pixel, np.float32),
                c(ph.dither_state, np.float32), c(ph.support_orders, np.int8), c(ph.pulse_height, np.int16),
                c(ph.u_pixel, np.float32), c(ph.v_pixel, np.float32), c(ph.detector_region, np.uint8),
                c(ph.pi, np.float32)]
        r = f(path.encode(), ph.n, *[_p(a) for a in cols], history, 1 if new else 0, total_time)
        if r != 0:
            raise RuntimeError("reference ray-file writer failed: " + self.lib.mxref_last_error().decode())

    def write_photons(self, ph: PhotonList, history: int, write_mask: int, out_dir: str, new: bool = True,
                      total_time: float = 0.0):
        """The reference's marx_write_photons over ph (host columns)."""
        c = lambda a, dt: np.ascontiguousarray(a, dtype=dt)
        f = self.lib.mxref_write_photons
        f.argtypes = [C.c_char_p, C.c_int] + [C.c_void_p] * 17 + [C.c_ulong, C.c_ulong, C.c_int, C.c_double]
        cols = [c(ph.energy, np.float64), c(ph.x, np.float64), c(ph.p, np.float64), c(ph.arrival_time, np.float64),
                c(ph.flags, np.uint32), c(ph.tag, np.uint32), c(ph.mirror_shell, np.int8), c(ph.order, np.int8),
                c(ph.ccd_num, np.int8), c(ph.y_pixel, np.float32), c(ph.z_pixel, np.float32),
                c(ph.dither_state, np.float32), c(ph.support_orders, np.int8), c(ph.pulse_height, np.int16),
                c(ph.u_pixel, np.float32), c(ph.v_pixel, np.float32), c(ph.detector_region, np.uint8)]
        r = f(out_dir.encode(), ph.n, *[_p(a) for a in cols], history, write_mask, 1 if new else 0, total_time)
        if r != 0:
            raise RuntimeError("reference writer failed: " + self.lib.mxref_last_error().decode())

    def source_photons(self, n: int, U=None, direction=None):
        """(source direction st->p, energies, directions (3, n)) of n photons
        of the source the parameters describe, one create_photons call per
        photon; U (4, n) slot-major uniforms for the slot build; direction
        replaces st->p after the source's set-up."""
        p0 = np.zeros(3)
        if self.lib.mxref_source_setup(_p(p0)) != 0:
            raise RuntimeError("reference source: " + self.lib.mxref_last_error().decode())
        if direction is not None:
            p0 = np.ascontiguousarray(direction, dtype=np.float64)
            if self.lib.mxref_source_set_direction(_p(p0)) != 0:
                raise RuntimeError("reference source: " + self.lib.mxref_last_error().decode())
        e = np.zeros(n)
        p = np.zeros((n, 3))
        Up = np.ascontiguousarray(U.T) if U is not None else np.zeros((n, 4))
        if self.lib.mxref_source_photons(n, _p(Up), _p(e), _p(p)) != 0:
            raise RuntimeError("reference source photons: " + self.lib.mxref_last_error().decode())
        return p0, e, np.ascontiguousarray(p.T)

    def source_batch(self, n: int, U=None):
        """One create_photons call of up to n photons of the source set up
        by source_photons or source_open (U: the uniforms in draw order).
        Returns a PhotonList of the photons made (energy, x, p, arrival time,
        flags, mirror shell), with the count of uniforms drawn as
        uniforms_used."""
        e, t = np.zeros(n), np.zeros(n)
        x, p = np.zeros((n, 3)), np.zeros((n, 3))
        flags, shell = np.zeros(n, np.uint32), np.zeros(n, np.int32)
        num, used = C.c_uint(0), C.c_int(0)
        u = np.ascontiguousarray(U if U is not None else np.zeros(0), dtype=np.float64)
        if self.lib.mxref_source_batch(n, _p(u), u.size, _p(e), _p(x), _p(p), _p(t), _p(flags), _p(shell),
                                       C.byref(num), C.byref(used)) != 0:
            raise RuntimeError("reference source batch: " + self.lib.mxref_last_error().decode())
        m = num.value
        q = PhotonList(m)
        q.energy[:] = e[:m]; q.arrival_time[:] = t[:m]; q.flags[:] = flags[:m]
        q.x[:] = x[:m].T; q.p[:] = p[:m].T; q.mirror_shell[:] = shell[:m]
        q.uniforms_used = used.value
        return q

    def source_open(self):
        """Set up and open the source the parameters describe."""
        p0 = np.zeros(3)
        if self.lib.mxref_source_setup(_p(p0)) != 0:
            raise RuntimeError("reference source: " + self.lib.mxref_last_error().decode())
        return p0

    def trace_batch(self, ph: PhotonList, stages: int = 15):
        """Whole batch with the reference's own generator; returns (list, seconds)."""
        assert self.native
        n = ph.n
        E = np.ascontiguousarray(ph.energy); P = np.ascontiguousarray(ph.p.T); T = np.ascontiguousarray(ph.arrival_time)
        o = self._outs(n)
        f = self.lib.mxref_trace_batch
        f.restype = C.c_double
        secs = f(n, _p(E), _p(P), _p(T), stages, _p(o["x"]), _p(o["p"]), _p(o["flags"]), _p(o["shell"]),
                 _p(o["order"]), _p(o["ccd"]), _p(o["ypix"]), _p(o["zpix"]), _p(o["dith"]))
        if secs < 0:
            raise RuntimeError("reference batch trace failed")
        return self._to_list(ph, o), secs
