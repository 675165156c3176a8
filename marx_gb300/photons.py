"""Structure-of-arrays photon list (``mx_photons`` in include/marx_gb300.h).

The reference keeps photons as an array of 136-byte structs
(``Marx_Photon_Attr_Type``, marx/libsrc/marx.h:51-100).  Here each attribute
is its own contiguous column so that a warp reads 32 consecutive values per
load; 3-vectors are stored component-major (all x, then all y, then all z).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

# flag bits, marx.h:65-75
PHOTON_UNDETECTED = 0x01
PHOTON_UNREFLECTED = 0x02
PHOTON_UNDIFFRACTED = 0x04
PHOTON_MISSED_DETECTOR = 0x08
PHOTON_MIRROR_VBLOCKED = 0x10
PHOTON_GRATING_VBLOCKED = 0x40
BAD_PHOTON_MASK = 0xFF
PHOTON_DRAKE_BLOCKED = 0x20
PHOTON_DRAKE_REFLECTED = 0x100
PHOTON_ACIS_STREAKED = 0x200
PHOTON_VARIATE_OVERRUN = 0x10000

STAGE_DITHER, STAGE_MIRROR, STAGE_GRATING, STAGE_DETECT = 1, 2, 4, 8
STAGE_ALL = 15
NUM_U, NUM_N = 36, 24


class MxPhotons(C.Structure):
    _fields_ = [
        ("n", C.c_uint32), ("stride", C.c_uint32),
        ("energy", C.c_void_p), ("x", C.c_void_p), ("p", C.c_void_p),
        ("arrival_time", C.c_void_p), ("flags", C.c_void_p), ("tag", C.c_void_p),
        ("mirror_shell", C.c_void_p), ("order", C.c_void_p), ("ccd_num", C.c_void_p),
        ("reserved8", C.c_void_p),
        ("y_pixel", C.c_void_p), ("z_pixel", C.c_void_p), ("dither_state", C.c_void_p),
        ("support_orders", C.c_void_p), ("pulse_height", C.c_void_p), ("u_pixel", C.c_void_p),
        ("v_pixel", C.c_void_p), ("detector_region", C.c_void_p), ("pi", C.c_void_p),
        ("det_dither", C.c_void_p),
    ]


class MxVariates(C.Structure):
    _fields_ = [("U", C.c_void_p), ("N", C.c_void_p)]


COLUMNS = {
    # name: (dtype, components)
    "energy": (np.float64, 1), "x": (np.float64, 3), "p": (np.float64, 3),
    "arrival_time": (np.float64, 1), "flags": (np.uint32, 1), "tag": (np.uint32, 1),
    "mirror_shell": (np.int8, 1), "order": (np.int8, 1), "ccd_num": (np.int8, 1),
    "y_pixel": (np.float32, 1), "z_pixel": (np.float32, 1), "dither_state": (np.float32, 3),
    "support_orders": (np.int8, 4), "pulse_height": (np.int16, 1), "u_pixel": (np.float32, 1),
    "v_pixel": (np.float32, 1), "detector_region": (np.uint8, 1), "pi": (np.float32, 1),
}
# Columns a list carries only when asked for (None otherwise): the detector
# dither dy, dz, dtheta, non-zero with DitherModel FILE only.
OPTIONAL_COLUMNS = {"det_dither": (np.float32, 3)}


class PhotonList:
    """Host photon list: one numpy column per attribute."""

    def __init__(self, n: int, det_dither: bool = False):
        self.n = int(n)
        for k, (dt, m) in COLUMNS.items():
            shape = (m, self.n) if m > 1 else (self.n,)
            setattr(self, k, np.zeros(shape, dtype=dt))
        self.det_dither = np.zeros((3, self.n), np.float32) if det_dither else None
        self.ccd_num[:] = -1
        self.tag[:] = np.arange(self.n, dtype=np.uint32)

    @classmethod
    def from_inputs(cls, energy, p, arrival_time=None, tag=None):
        ph = cls(len(energy))
        ph.energy[:] = energy
        ph.p[:] = np.asarray(p).reshape(3, -1) if np.asarray(p).shape[0] == 3 else np.asarray(p).T
        if arrival_time is not None:
            ph.arrival_time[:] = arrival_time
        if tag is not None:
            ph.tag[:] = tag
        return ph

    def copy(self) -> "PhotonList":
        q = PhotonList.__new__(PhotonList)
        q.n = self.n
        for k in COLUMNS:
            setattr(q, k, getattr(self, k).copy())
        dd = getattr(self, "det_dither", None)
        q.det_dither = None if dd is None else dd.copy()
        return q

    def struct(self) -> MxPhotons:
        s = MxPhotons()
        s.n = self.n
        for k in list(COLUMNS) + list(OPTIONAL_COLUMNS):
            a = getattr(self, k, None)
            if a is None:
                continue
            assert a.flags["C_CONTIGUOUS"]
            setattr(s, k, a.ctypes.data)
        return s

    def good(self) -> np.ndarray:
        return (self.flags & BAD_PHOTON_MASK) == 0

    def nbytes_inputs(self) -> int:
        return self.energy.nbytes + self.p.nbytes + self.arrival_time.nbytes + self.tag.nbytes


def predraw_variates(n: int, seed: int):
    """Independent per-photon uniforms in [0,1) and unit normals, slot-major."""
    rng = np.random.default_rng(seed)
    U = np.ascontiguousarray(rng.random((NUM_U, n)))
    N = np.ascontiguousarray(rng.standard_normal((NUM_N, n)))
    return U, N
