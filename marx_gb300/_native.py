"""ctypes binding of libmarx_gb300.so (the C ABI in include/marx_gb300.h).

There is no fallback: if the library is missing or no CUDA device is
present, constructing an Engine raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .config import MxConfig
from .photons import COLUMNS, OPTIONAL_COLUMNS, MxPhotons, MxVariates, PhotonList, NUM_U, NUM_N

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmarx_gb300.so")

SYMBOLS = [
    "mx_config_default", "mx_create", "mx_configure", "mx_destroy", "mx_last_error", "mx_trace",
    "mx_trace_host", "mx_compact", "mx_table_bytes", "mx_launch_count", "mx_validate_config",
    "mx_stream", "mx_overrun_count", "mx_probe_fp64", "mx_set_trace_mode",
]
MODE_AUTO, MODE_FUSED, MODE_WAVEFRONT = 0, 1, 2

_lib = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is not built; run `python -m marx_gb300.build`")
    L = C.CDLL(path)
    L.mx_config_default.argtypes = [C.POINTER(MxConfig)]
    L.mx_create.restype = C.c_void_p
    L.mx_create.argtypes = [C.c_char_p, C.POINTER(MxConfig)]
    L.mx_configure.argtypes = [C.c_void_p, C.POINTER(MxConfig)]
    L.mx_validate_config.argtypes = [C.c_char_p, C.POINTER(MxConfig)]
    L.mx_destroy.argtypes = [C.c_void_p]
    L.mx_last_error.restype = C.c_char_p
    L.mx_last_error.argtypes = [C.c_void_p]
    L.mx_trace.argtypes = [C.c_void_p, C.POINTER(MxPhotons), C.c_uint32, C.POINTER(MxVariates), C.c_uint64, C.c_void_p]
    L.mx_trace_host.argtypes = [C.c_void_p, C.POINTER(MxPhotons), C.c_uint32, C.POINTER(MxVariates), C.c_uint64]
    L.mx_compact.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(C.c_uint32), C.c_void_p]
    L.mx_table_bytes.argtypes = [C.c_void_p, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
    L.mx_launch_count.restype = C.c_uint64
    L.mx_launch_count.argtypes = [C.c_void_p]
    L.mx_stream.restype = C.c_void_p
    L.mx_stream.argtypes = [C.c_void_p]
    L.mx_overrun_count.argtypes = [C.c_void_p, C.POINTER(C.c_ulonglong), C.c_int]
    L.mx_probe_fp64.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.mx_set_trace_mode.argtypes = [C.c_void_p, C.c_int]
    L.mx_set_aspect_solution.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                         C.c_double, C.c_int]
    _lib = L
    return L


class DevicePhotons:
    """Photon list resident on the GPU: one torch tensor per column."""

    def __init__(self, n: int, device="cuda", det_dither: bool = False):
        import torch
        self.n = int(n)
        tmap = {np.float64: torch.float64, np.float32: torch.float32, np.uint32: torch.int32,
                np.int8: torch.int8, np.int16: torch.int16, np.uint8: torch.uint8}
        for k, (dt, m) in COLUMNS.items():
            shape = (m, self.n) if m > 1 else (self.n,)
            setattr(self, k, torch.zeros(shape, dtype=tmap[dt], device=device))
        self.det_dither = torch.zeros((3, self.n), dtype=torch.float32, device=device) if det_dither else None
        self.ccd_num.fill_(-1)

    @classmethod
    def from_host(cls, ph: PhotonList, device="cuda"):
        import torch
        d = cls.__new__(cls)
        d.n = ph.n
        for k in COLUMNS:
            a = getattr(ph, k)
            if a.dtype == np.uint32:
                a = a.view(np.int32)
            setattr(d, k, torch.from_numpy(np.ascontiguousarray(a)).to(device))
        dd = getattr(ph, "det_dither", None)
        d.det_dither = None if dd is None else torch.from_numpy(np.ascontiguousarray(dd)).to(device)
        return d

    def to_host(self) -> PhotonList:
        q = PhotonList.__new__(PhotonList)
        q.n = self.n
        for k, (dt, m) in COLUMNS.items():
            a = getattr(self, k).cpu().numpy()
            setattr(q, k, a.view(dt) if a.dtype != dt else a)
        dd = getattr(self, "det_dither", None)
        q.det_dither = None if dd is None else dd.cpu().numpy()
        return q

    def struct(self) -> MxPhotons:
        s = MxPhotons()
        s.n = self.n
        for k in list(COLUMNS) + list(OPTIONAL_COLUMNS):
            t = getattr(self, k, None)
            if t is None:
                continue
            assert t.is_contiguous()
            setattr(s, k, t.data_ptr())
        return s


class Engine:
    """One mx_context: model tables resident on the current CUDA device."""

    def __init__(self, cfg: MxConfig, pack: str | None = None):
        self.lib = load_library()
        if pack is None:
            from .caldb.pack import DEFAULT_PACK
            pack = DEFAULT_PACK
        self.cfg = cfg
        self.h = self.lib.mx_create(pack.encode(), C.byref(cfg))
        if not self.h:
            raise RuntimeError("mx_create: " + self.lib.mx_last_error(None).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.mx_destroy(self.h)
            self.h = None

    __del__ = close

    def _check(self, r):
        if r != 0:
            raise RuntimeError(f"marx_gb300 error {r}: " + self.lib.mx_last_error(self.h).decode())

    def set_aspect_solution(self, asp, record_only: bool = False):
        """DitherModel FILE: the aspect solution (an ``AspectSolution``, see
        ``marx_gb300.aspsol``) for the dither and detector stages
        (mx_set_aspect_solution); None removes it."""
        if asp is None:
            self._check(self.lib.mx_set_aspect_solution(self.h, None, 0, 0.0, 0.0, 0.0, 0.0, 0))
            return
        rows = np.ascontiguousarray(asp.rows, dtype=np.float64)
        assert rows.ndim == 2 and rows.shape[1] == 7
        self._check(self.lib.mx_set_aspect_solution(self.h, rows.ctypes.data, rows.shape[0], asp.ra_nom, asp.dec_nom,
                                                    asp.roll_nom, asp.tstart, 1 if record_only else 0))

    def set_mode(self, mode: int):
        """MODE_AUTO, MODE_FUSED or MODE_WAVEFRONT (include/marx_gb300.h)."""
        self._check(self.lib.mx_set_trace_mode(self.h, mode))

    def configure(self, cfg: MxConfig):
        self._check(self.lib.mx_configure(self.h, C.byref(cfg)))
        self.cfg = cfg

    def set_start_time(self, start_time: float):
        """Marx_Photon_Type.start_time of the photons traced next
        (mx_set_start_time)."""
        self.lib.mx_set_start_time.argtypes = [C.c_void_p, C.c_double]
        self._check(self.lib.mx_set_start_time(self.h, float(start_time)))

    def trace(self, ph: DevicePhotons, stages: int = 15, U=None, N=None, seed: int = 0, stream=None):
        """In-place trace of device photons (U, N: device tensors or None)."""
        s = ph.struct()
        v = MxVariates(U.data_ptr() if U is not None else None, N.data_ptr() if N is not None else None)
        st = stream.cuda_stream if stream is not None else self.current_stream()
        self._check(self.lib.mx_trace(self.h, C.byref(s), stages, C.byref(v), seed, C.c_void_p(st)))

    @staticmethod
    def current_stream():
        import torch
        return torch.cuda.current_stream().cuda_stream

    def trace_host(self, ph: PhotonList, stages: int = 15, U=None, N=None, seed: int = 0):
        """Blocking trace of host photons: copies in, traces, copies back."""
        s = ph.struct()
        v = MxVariates(U.ctypes.data if U is not None else None, N.ctypes.data if N is not None else None)
        self._check(self.lib.mx_trace_host(self.h, C.byref(s), stages, C.byref(v), seed))

    def compact(self, flags, stream=None):
        """Indices (device int32 tensor) of photons without a bad flag."""
        import torch
        n = flags.numel()
        idx = torch.empty(n, dtype=torch.int32, device=flags.device)
        cnt = C.c_uint32(0)
        st = stream.cuda_stream if stream is not None else self.current_stream()
        self._check(self.lib.mx_compact(self.h, C.c_void_p(flags.data_ptr()), n, C.c_void_p(idx.data_ptr()),
                                        C.byref(cnt), C.c_void_p(st)))
        return idx[:cnt.value]

    def table_bytes(self):
        a, b = C.c_size_t(0), C.c_size_t(0)
        self._check(self.lib.mx_table_bytes(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def launch_count(self) -> int:
        return int(self.lib.mx_launch_count(self.h))

    def overrun_count(self, reset=True) -> int:
        c = C.c_ulonglong(0)
        self._check(self.lib.mx_overrun_count(self.h, C.byref(c), 1 if reset else 0))
        return c.value

    def stream_handle(self) -> int:
        return self.lib.mx_stream(self.h)


def validate_config(cfg: MxConfig, pack: str | None = None) -> str | None:
    """None if the configuration is usable, else the reason (no GPU needed)."""
    L = load_library()
    if pack is None:
        from .caldb.pack import DEFAULT_PACK
        pack = DEFAULT_PACK
    r = L.mx_validate_config(pack.encode(), C.byref(cfg))
    return None if r == 0 else L.mx_last_error(None).decode()


def probe_fp64():
    """Measured FP64 FMA throughput (TFLOP/s) of the current device."""
    L = load_library()
    t, ms = C.c_double(0), C.c_double(0)
    if L.mx_probe_fp64(C.byref(t), C.byref(ms)) != 0:
        raise RuntimeError("FP64 probe failed")
    return t.value
