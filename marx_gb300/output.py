"""MARX output directories: one big-endian column file per photon attribute.

``write_photons`` is the C ABI's ``mx_write_photons`` (the reference's
marx_write_photons, marx/libsrc/marxio.c:395-478); ``read_column`` and
``read_dir`` read such files back (any MARX output directory).
"""
from __future__ import annotations

import ctypes as C
import os
import struct

import numpy as np

from .config import MxConfig
from .photons import PhotonList

# MX_OUT_* (include/marx_gb300.h), the reference's MARX_*_OK history bits
OUT = {"ENERGY": 0x1, "TIME": 0x2, "X": 0x4, "P": 0x8, "TAG": 0x10, "PHA": 0x20, "PI": 0x40, "DET_PIXEL": 0x80,
       "DET_NUM": 0x100, "DET_REGION": 0x200, "DET_UV": 0x400, "SHELL": 0x800, "SKY_DITHER": 0x1000,
       "DET_DITHER": 0x2000, "ORDER": 0x100000, "ORDER1": 0x200000, "ORDER2": 0x400000, "ORDER3": 0x800000,
       "ORDER4": 0x1000000}
ALL = sum(OUT.values())
_TYPES = {b"E": ">f4", b"J": ">i4", b"I": ">i2", b"A": "i1", b"F": ">f8"}


def _lib():
    from ._native import load_library
    L = load_library()
    if not getattr(L, "_mx_output_bound", False):
        from .photons import MxPhotons
        L.mx_write_photons.argtypes = [C.POINTER(MxPhotons), C.c_uint32, C.c_uint32, C.c_int, C.c_char_p, C.c_int,
                                       C.c_double]
        L.mx_write_error.restype = C.c_char_p
        L.mx_output_history.restype = C.c_uint32
        L.mx_output_history.argtypes = [C.POINTER(MxConfig), C.c_uint32]
        L._mx_output_bound = True
    return L


def history(cfg: MxConfig, stages: int = 15) -> int:
    """The history bits a trace of cfg through `stages` makes valid."""
    return int(_lib().mx_output_history(C.byref(cfg), stages))


def write_photons(ph: PhotonList, hist: int, write_mask: int, out_dir: str, append: bool = False,
                  total_time: float = 0.0, dither: bool = True) -> None:
    os.makedirs(out_dir, exist_ok=True)
    L = _lib()
    s = ph.struct()
    r = L.mx_write_photons(C.byref(s), hist, write_mask, 1 if dither else 0, out_dir.encode(), 1 if append else 0,
                           total_time)
    if r != 0:
        raise RuntimeError("mx_write_photons: " + L.mx_write_error().decode())


def read_column(path: str):
    """(column name, values) of one column file."""
    b = open(path, "rb").read()
    if b[:4] != bytes([0x83, 0x13, 0x89, 0x8D]):
        raise ValueError(f"{path}: not a MARX column file")
    name = b[5:20].split(b"\0")[0].decode()
    rows = struct.unpack(">i", b[20:24])[0]
    dt = np.dtype(_TYPES[b[4:5]])
    return name, np.frombuffer(b, dtype=dt, count=rows, offset=32).astype(dt.newbyteorder("="))


def read_dir(out_dir: str) -> dict:
    """Every column file of an output directory: {file stem: values}."""
    out = {}
    for f in sorted(os.listdir(out_dir)):
        if f.endswith(".dat"):
            out[f[:-4]] = read_column(os.path.join(out_dir, f))[1]
    return out
