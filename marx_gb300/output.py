"""MARX output directories: one big-endian column file per photon attribute.

``write_photons`` is the C ABI's ``mx_write_photons`` (the reference's
marx_write_photons, marx/libsrc/marxio.c:395-478); ``read_column`` and
``read_dir`` read such files back (any MARX output directory);
``write_run_files`` adds the marx.par and obs.par that marx2fits reads
beside the column files.
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


def _ray_lib():
    L = _lib()
    if not getattr(L, "_mx_ray_bound", False):
        from .photons import MxPhotons
        L.mx_write_rayfile.argtypes = [C.POINTER(MxPhotons), C.c_uint64, C.c_char_p, C.c_int, C.c_double]
        L.mx_read_rayfile.argtypes = [C.c_char_p, C.POINTER(MxPhotons), C.c_uint32, C.POINTER(C.c_uint64),
                                      C.POINTER(C.c_double), C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]
        L._mx_ray_bound = True
    return L


def write_rayfile(ph: PhotonList, hist: int, path: str, append: bool = False, total_time: float = 0.0) -> None:
    """MARX's ray file of the photons without a bad flag (mx_write_rayfile;
    marx_dump_to_rayfile, marx/libsrc/s-rayfile.c:109-155)."""
    L = _ray_lib()
    s = ph.struct()
    if L.mx_write_rayfile(C.byref(s), hist, path.encode(), 1 if append else 0, total_time) != 0:
        raise RuntimeError("mx_write_rayfile: " + L.mx_write_error().decode())


def read_rayfile(path: str, batch: int | None = None):
    """The photons of a ray file as PhotonLists of at most `batch` photons
    (all at once by default), with the RAYFILE source's arrival times: each
    batch's times relative to the last photon of the batch before
    (rayfile_create_photons, s-rayfile.c:188-219).  Returns (history, lists)."""
    L = _ray_lib()
    n_all = max(0, (os.path.getsize(path) - 2 * C.sizeof(C.c_ulong)) // 136)
    batch = batch or max(1, n_all)
    off, last, hist, got = C.c_uint64(0), C.c_double(0.0), C.c_uint64(0), C.c_uint32(0)
    out = []
    while True:
        ph = PhotonList(batch, det_dither=True)
        s = ph.struct()
        if L.mx_read_rayfile(path.encode(), C.byref(s), batch, C.byref(off), C.byref(last), C.byref(hist),
                             C.byref(got)) != 0:
            raise RuntimeError("mx_read_rayfile: " + L.mx_write_error().decode())
        if got.value == 0:
            break
        q = PhotonList(got.value)
        for k in vars(ph):
            if k != "n" and getattr(ph, k) is not None:
                setattr(q, k, np.ascontiguousarray(getattr(ph, k)[..., :got.value]))
        out.append(q)
    return hist.value, out


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


def _par_lines(text: str):
    return [ln for ln in text.splitlines() if ln.strip()]   # pfile reading stops at a blank line


def _value_span(ln: str):
    """Start and end of the value field (the fourth) of a .par line."""
    pos = 0
    for _ in range(3):
        pos = ln.index(",", pos) + 1
    if ln[pos:pos + 1] == '"':
        end = ln.index('"', pos + 1) + 1
    else:
        end = ln.find(",", pos)
        end = len(ln) if end < 0 else end
    return pos, end


def _par_set(lines, name, value, kind="r"):
    """Set the value of parameter `name` (names compare without case, as
    pfile's do); append a hidden parameter when the file lacks it."""
    for i, ln in enumerate(lines):
        if ln.startswith("#") or ln.count(",") < 3:
            continue
        if ln.split(",", 1)[0].strip().lower() == name.lower():
            quoted = ln.split(",", 2)[1].strip()[:1] in ("s", "f")
            a, b = _value_span(ln)
            lines[i] = ln[:a] + (f'"{value}"' if quoted else str(value)) + ln[b:]
            return
    v = f'"{value}"' if kind in ("s", "f") else str(value)
    lines.append(f'{name},{kind},h,{v},,,""')


def write_run_files(out_dir: str, cfg: MxConfig, par_template: str, data_dir: str, total_time: float,
                    source_name: str = "POINT") -> None:
    """marx.par and obs.par of a run, so that marx2fits, marxcat and the
    other readers take the output directory as marx's own: the user's
    parameter file with the configuration's values (marx copies it,
    marx.c:475-503), and the detector's observation template from the MARX
    data directory (obs/<detector>_obs.par) with the pointing, instrument,
    focal length, offsets and times write_obs_par learns into it
    (marx.c:999-1196; the dither averages, zero for INTERNAL dither, and the
    calendar dates from TStart are left at the template's)."""
    from .config import to_par
    os.makedirs(out_dir, exist_ok=True)
    lines = _par_lines(open(par_template).read())
    names = {ln.split(",", 1)[0].strip().lower() for ln in lines if not ln.startswith("#")}
    for k, v in to_par(cfg).items():
        if k.lower() in names:
            _par_set(lines, k, v)
    with open(os.path.join(out_dir, "marx.par"), "w") as fh:
        fh.write("\n".join(lines) + "\n")
    det = {1: "ACIS-I", 2: "ACIS-S", 3: "HRC-I", 4: "HRC-S"}.get(int(cfg.detector), "NONE")
    grat = {1: "HETG", 2: "LETG"}.get(int(cfg.grating), "NONE")
    tmpl = {"ACIS-I": "acis_i_obs.par", "ACIS-S": "acis_s_obs.par", "HRC-I": "hrc_i_obs.par",
            "HRC-S": "hrc_s_obs.par"}.get(det, "generic_obs.par")
    obs = _par_lines(open(os.path.join(data_dir, "obs", tmpl)).read())
    norm = lambda a: a % 360.0
    datamode = "GRADED" if det.startswith("ACIS") else ("SPECTROSCOPIC" if grat != "NONE" else "IMAGING")
    for k, v, kind in (("ra_nom", norm(cfg.ra_nom), "r"), ("roll_nom", norm(cfg.roll_nom), "r"),
                       ("dec_nom", cfg.dec_nom, "r"), ("ra_pnt", norm(cfg.ra_nom), "r"),
                       ("roll_pnt", norm(cfg.roll_nom), "r"), ("dec_pnt", cfg.dec_nom, "r"),
                       ("foc_len", cfg.focal_length, "r"), ("datamode", datamode, "s"), ("detnam", det, "s"),
                       ("grating", grat, "s"), ("object", source_name, "s"), ("title", source_name, "s"),
                       ("tstart", 0.0, "r"), ("tstop", total_time, "r"),
                       ("sim_x", cfg.det_offset[0], "r"), ("sim_y", cfg.det_offset[1], "r"),
                       ("sim_z", cfg.det_offset[2], "r"), ("defocus", cfg.det_offset[0], "r"),
                       ("DY_AVG", 0.0, "r"), ("DZ_AVG", 0.0, "r"), ("DTH_AVG", 0.0, "r"),
                       ("LIVETIME", total_time, "r"), ("ONTIME", total_time, "r"),
                       ("EXPOSURE", total_time, "r"), ("TELAPSE", total_time, "r")):
        _par_set(obs, k, repr(float(v)) if kind == "r" else v, kind)
    with open(os.path.join(out_dir, "obs.par"), "w") as fh:
        fh.write("\n".join(obs) + "\n")
