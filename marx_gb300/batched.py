"""Batched form: many point sources in one persistent launch (mx_batch_* in
include/marx_gb300.h), and the 256-source workload.

    eng = Engine(batched_config())
    b = Batch(eng, batched_sources())
    b.tune()                      # autotuner, remembered per batch hash
    b.run(seed)                   # one CUDA-graph launch
    ph = b.photons()              # device columns (torch views)
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from .config import MxConfig, default_config, DETECTOR, GRATING, DITHER
from .photons import COLUMNS, MxPhotons

ARCMIN = math.pi / (180.0 * 60.0)


class MxSource(C.Structure):
    _fields_ = [("p", C.c_double * 3), ("energy_min", C.c_double), ("energy_max", C.c_double),
                ("num_photons", C.c_uint32), ("grating", C.c_int32), ("detector", C.c_int32),
                ("reserved", C.c_uint32), ("kind", C.c_int32), ("spectrum_n", C.c_uint32),
                ("param", C.c_double * 4), ("spectrum_energy", C.c_void_p), ("spectrum_flux", C.c_void_p),
                ("image_nx", C.c_uint32), ("image_ny", C.c_uint32), ("image", C.c_void_p)]


# source models (MX_SOURCE_* in include/marx_gb300.h) and their parameters
SOURCE = {"POINT": 0, "GAUSS": 1, "BETA": 2, "DISK": 3, "LINE": 4, "IMAGE": 5}


def make_source(p, kind="POINT", param=(), energy=(1.0, 1.0), spectrum=None, num_photons=0,
                grating="NONE", detector="ACIS-I", image=None) -> MxSource:
    """One source: p the unit direction of travel, kind and param as
    mx_source documents them, a FLAT spectrum (energy_min, energy_max) or a
    FILE spectrum (energies, flux), and for an IMAGE source the pixel array
    (NAXIS2 rows of NAXIS1, e.g. from ``read_image_fits``) with param the
    degrees per pixel; the returned struct references the arrays (keep it
    alive while it is used)."""
    s = MxSource()
    s.p[:] = list(p)
    s.kind = SOURCE[kind]
    for k, v in enumerate(param):
        s.param[k] = v
    s.energy_min, s.energy_max = energy
    s.num_photons = int(num_photons)
    s.grating, s.detector = GRATING[grating], DETECTOR[detector]
    if spectrum is not None:
        e = np.ascontiguousarray(spectrum[0], dtype=np.float64)
        f = np.ascontiguousarray(spectrum[1], dtype=np.float64)
        s._keep = (e, f)
        s.spectrum_n = len(e)
        s.spectrum_energy, s.spectrum_flux = e.ctypes.data, f.ctypes.data
    if image is not None:
        im = np.ascontiguousarray(image, dtype=np.float32)
        s._keep_image = im
        s.image_ny, s.image_nx = im.shape
        s.image = im.ctypes.data
    return s


def read_image_fits(path: str):
    """The primary image of a FITS file as the IMAGE source reads it
    (open_image_fits_file and read_image, s-image.c:46-232): pixel values as
    float32 (BITPIX 8, 16, 32, -32 or -64; no BSCALE/BZERO), and the degrees
    per pixel from CDELT1/CDELT2, else the CD matrix, else (0, 0) for the
    model's 0.5 arcsec default.  Returns (image[NAXIS2, NAXIS1], (s1, s2))."""
    b = open(path, "rb").read()
    hdr, off = {}, 0
    while True:
        blk = b[off:off + 2880]
        if len(blk) < 2880:
            raise ValueError(f"{path}: truncated FITS header")
        off += 2880
        done = False
        for i in range(36):
            card = blk[i * 80:(i + 1) * 80].decode("ascii", "replace")
            key = card[:8].strip()
            if key == "END":
                done = True
                break
            if card[8:10] == "= ":
                hdr[key] = card[10:].split("/")[0].strip()
        if done:
            break
    nx, ny, bitpix = int(hdr["NAXIS1"]), int(hdr["NAXIS2"]), int(hdr["BITPIX"])
    dt = {8: ">u1", 16: ">i2", 32: ">i4", -32: ">f4", -64: ">f8"}.get(bitpix)
    if dt is None:
        raise ValueError(f"BITPIX = {bitpix} is not supported")
    img = np.frombuffer(b, dtype=dt, count=nx * ny, offset=off).astype(np.float32).reshape(ny, nx)
    num = lambda k: float(hdr[k].replace("D", "E"))
    if "CDELT1" in hdr:
        s1, s2 = abs(num("CDELT1")), abs(num("CDELT2"))
    elif "CD1_1" in hdr:
        a, b2, c, d = num("CD1_1"), num("CD1_2"), num("CD2_1"), num("CD2_2")
        s1 = math.sqrt(a * a + b2 * b2)
        s2 = math.sqrt(c * c + d * d)
    else:
        s1 = s2 = 0.0
    return img, (s1, s2)


class MxBatchParams(C.Structure):
    _fields_ = [("block", C.c_int32), ("tile", C.c_int32), ("blocks_per_sm", C.c_int32), ("reserved", C.c_int32)]

    def as_dict(self):
        return {"block": self.block, "tile": self.tile, "blocks_per_sm": self.blocks_per_sm}


def batched_config() -> MxConfig:
    """Mirror with blur, WFold scattering and struts; no dither (each
    source's direction is given); per-source grating and detector."""
    c = default_config()
    c.dither = DITHER["NONE"]
    c.roll_nom = 0.0
    c.grating = GRATING["NONE"]
    c.detector = DETECTOR["ACIS-I"]
    return c


def batched_sources(nsrc: int = 256, seed: int = 404, nmin: float = 1e3, nmax: float = 1e6,
                    emin: float = 0.3, emax: float = 10.0, max_offaxis_arcmin: float = 10.0):
    """256 point sources: photon counts log-uniform in [nmin, nmax], off-axis
    angle uniform in [0, 10'] at uniform azimuth, energies uniform in
    [0.3, 10] keV, grating NONE or HETG and detector ACIS-I or ACIS-S drawn
    independently per source."""
    r = np.random.default_rng(seed)
    counts = np.exp(r.uniform(np.log(nmin), np.log(nmax), nsrc)).astype(np.int64)
    theta = r.uniform(0.0, max_offaxis_arcmin * ARCMIN, nsrc)
    phi = r.uniform(0.0, 2 * np.pi, nsrc)
    grat = r.integers(0, 2, nsrc)
    det = r.integers(0, 2, nsrc)
    arr = (MxSource * nsrc)()
    for s in range(nsrc):
        st = math.sin(theta[s])
        arr[s].p[:] = [-math.cos(theta[s]), st * math.cos(phi[s]), st * math.sin(phi[s])]
        arr[s].energy_min, arr[s].energy_max = emin, emax
        arr[s].num_photons = int(counts[s])
        arr[s].grating = GRATING["HETG"] if grat[s] else GRATING["NONE"]
        arr[s].detector = DETECTOR["ACIS-S"] if det[s] else DETECTOR["ACIS-I"]
    return arr


class _DevArray:
    """__cuda_array_interface__ view of a device pointer (no copy)."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"data": (int(ptr), False), "shape": tuple(shape),
                                         "typestr": typestr, "version": 3}


def bind(L):
    L.mx_batch_create.restype = C.c_void_p
    L.mx_batch_create.argtypes = [C.c_void_p, C.POINTER(MxSource), C.c_int]
    L.mx_batch_destroy.argtypes = [C.c_void_p]
    L.mx_batch_set_params.argtypes = [C.c_void_p, C.POINTER(MxBatchParams)]
    L.mx_batch_get_params.argtypes = [C.c_void_p, C.POINTER(MxBatchParams)]
    L.mx_batch_tune.argtypes = [C.c_void_p, C.c_int, C.POINTER(MxBatchParams)]
    L.mx_batch_run.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p]
    L.mx_batch_run_sequential.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p]
    L.mx_batch_photons.argtypes = [C.c_void_p, C.POINTER(MxPhotons), C.POINTER(C.POINTER(C.c_uint32))]
    L.mx_batch_total_photons.restype = C.c_uint64
    L.mx_batch_total_photons.argtypes = [C.c_void_p]
    L.mx_generate_source.argtypes = [C.c_void_p, C.POINTER(MxSource), C.c_uint32, C.c_uint64,
                                     C.POINTER(MxPhotons), C.c_void_p]


class Batch:
    def __init__(self, engine, sources):
        self.eng = engine
        self.L = engine.lib
        bind(self.L)
        self.sources = sources
        self.h = self.L.mx_batch_create(engine.h, sources, len(sources))
        if not self.h:
            raise RuntimeError("mx_batch_create: " + self.L.mx_last_error(None).decode())
        self.n = int(self.L.mx_batch_total_photons(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.L.mx_batch_destroy(self.h)
            self.h = None

    __del__ = close

    def tune(self, trials: int = 2) -> dict:
        p = MxBatchParams()
        self.eng._check(self.L.mx_batch_tune(self.h, trials, C.byref(p)))
        return p.as_dict()

    def params(self) -> dict:
        p = MxBatchParams()
        self.L.mx_batch_get_params(self.h, C.byref(p))
        return p.as_dict()

    def set_params(self, block, tile, blocks_per_sm):
        p = MxBatchParams(block, tile, blocks_per_sm, 0)
        self.eng._check(self.L.mx_batch_set_params(self.h, C.byref(p)))

    def run(self, seed: int = 0, stream=None):
        st = stream.cuda_stream if stream is not None else self.eng.current_stream()
        self.eng._check(self.L.mx_batch_run(self.h, seed, C.c_void_p(st)))

    def run_sequential(self, seed: int = 0, stream=None):
        st = stream.cuda_stream if stream is not None else self.eng.current_stream()
        self.eng._check(self.L.mx_batch_run_sequential(self.h, seed, C.c_void_p(st)))

    def source_start(self) -> np.ndarray:
        s = MxPhotons()
        st = C.POINTER(C.c_uint32)()
        self.L.mx_batch_photons(self.h, C.byref(s), C.byref(st))
        return np.ctypeslib.as_array(st, shape=(len(self.sources) + 1,)).copy()

    def photons(self):
        """Torch views of the batch's device columns (valid while the batch lives)."""
        import torch
        s = MxPhotons()
        st = C.POINTER(C.c_uint32)()
        self.L.mx_batch_photons(self.h, C.byref(s), C.byref(st))
        out = {}
        code = {np.float64: "<f8", np.float32: "<f4", np.uint32: "<i4", np.int8: "|i1"}
        for k, (dt, m) in COLUMNS.items():
            if not getattr(s, k):       # columns a batch does not carry (LETG, HRC outputs)
                continue
            shape = (m, self.n) if m > 1 else (self.n,)
            out[k] = torch.as_tensor(_DevArray(getattr(s, k), shape, code[dt]), device="cuda")
        return out

    def to_host(self):
        from .photons import PhotonList
        q = PhotonList.__new__(PhotonList)
        q.n = self.n
        for k, t in self.photons().items():
            a = t.cpu().numpy()
            dt = COLUMNS[k][0]
            setattr(q, k, a.view(dt) if a.dtype != dt else a.copy())
        return q


def generate_source(engine, src: MxSource, first_tag: int, seed: int, dev_photons, stream=None):
    """Fill a DevicePhotons with one source's photons (mx_generate_source)."""
    bind(engine.lib)
    s = dev_photons.struct()
    st = stream.cuda_stream if stream is not None else engine.current_stream()
    engine._check(engine.lib.mx_generate_source(engine.h, C.byref(src), first_tag, seed, C.byref(s), C.c_void_p(st)))


def main(argv=None):
    """Batched launches of the 256-source workload on the current GPU:
    python -m marx_gb300.batched [--nmax N] [--steps K] [--shape B T P]
    (sources of 1e3 .. N photons, log-uniform; the autotuner's launch shape
    unless one is given)."""
    import argparse
    import torch
    from ._native import Engine
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--nmax", type=float, default=1e6)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--shape", type=int, nargs=3, metavar=("BLOCK", "TILE", "PER_SM"),
                    help="launch shape instead of the autotuner's choice")
    a = ap.parse_args(argv)
    eng = Engine(batched_config())
    b = Batch(eng, batched_sources(nmax=a.nmax))
    if a.shape:
        b.set_params(*a.shape)
        p = b.params()
    else:
        p = b.tune(trials=1)
    for s in range(a.steps):
        b.run(seed=s)
    torch.cuda.synchronize()
    print(f"{b.n} photons per launch, launch shape {p}")


if __name__ == "__main__":
    main()
