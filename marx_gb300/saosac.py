"""The SAOSAC source (mx_saosac_* in include/marx_gb300.h): rays of an SAO
raytrace of the mirror read from a FITS RAYTRACE table (s-saosac.c).

    s = SaosacFile("rays.fits", cfg.hrma_cap_x)
    ph = s.read(100000, seed=3)         # a PhotonList, or None at the end
    eng.trace(DevicePhotons.from_host(ph), stages=STAGE_DITHER | STAGE_GRATING | STAGE_DETECT)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .photons import MxPhotons, PhotonList


def _lib():
    from ._native import load_library
    L = load_library()
    if not getattr(L, "_mx_saosac_bound", False):
        L.mx_saosac_open.restype = C.c_void_p
        L.mx_saosac_open.argtypes = [C.c_char_p, C.c_double]
        L.mx_saosac_read.argtypes = [C.c_void_p, C.POINTER(MxPhotons), C.c_uint32, C.c_void_p, C.c_uint64, C.c_uint32,
                                     C.POINTER(C.c_uint32)]
        L.mx_saosac_rows.restype = C.c_uint64
        L.mx_saosac_rows.argtypes = [C.c_void_p]
        L.mx_saosac_close.argtypes = [C.c_void_p]
        L._mx_saosac_bound = True
    return L


class SaosacFile:
    def __init__(self, path: str, hrma_cap_x: float):
        self.L = _lib()
        self.h = self.L.mx_saosac_open(path.encode(), hrma_cap_x)
        if not self.h:
            raise RuntimeError("mx_saosac_open: " + self.L.mx_last_error(None).decode())
        self.rows = int(self.L.mx_saosac_rows(self.h))
        self.next_tag = 0

    def read(self, n: int, u=None, seed: int = 0):
        """Up to n photons from the next rows (u: one uniform per row of the
        file, indexed by row; None: Philox draws of the row under seed)."""
        ph = PhotonList(n)
        s = ph.struct()
        got = C.c_uint32(0)
        ua = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        r = self.L.mx_saosac_read(self.h, C.byref(s), n, None if ua is None else ua.ctypes.data, seed,
                                  self.next_tag, C.byref(got))
        if r != 0:
            raise RuntimeError("mx_saosac_read: " + self.L.mx_last_error(None).decode())
        m = got.value
        if m == 0:
            return None
        self.next_tag += m
        q = PhotonList.__new__(PhotonList)
        q.n = m
        for k in vars(ph):
            a = getattr(ph, k)
            if k != "n" and a is not None:
                setattr(q, k, np.ascontiguousarray(a[..., :m]))
        q.det_dither = None
        return q

    def close(self):
        if getattr(self, "h", None):
            self.L.mx_saosac_close(self.h)
            self.h = None

    __del__ = close
