"""Event coordinates of marx2fits (CHIPX/CHIPY, EXPNO, FLTGRADE/GRADE,
TDETX/TDETY, DETX/DETY, sky X/Y) through the C ABI's ``mx_event_coords``.

``EventParams`` holds what marx2fits reads from marx.par and obs.par
(marx/src/marx2fits.c:2262-2282, 2947-2959); an event list is a dict of
columns named as the output-directory files (``ccd``, ``xpixel``,
``ypixel``, ``time``, ``sky_ra`` ... ``det_theta``, ``b_energy``).
``event_coords_host`` runs on host numpy arrays; ``event_coords`` on device
tensors (torch), for instance the columns of a traced photon list picked by
``Engine.compact``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

EDSER, RANDOMIZE, NONE, EXACT = 0, 1, 2, 3
PIXADJ = {"EDSER": EDSER, "RANDOMIZE": RANDOMIZE, "NONE": NONE, "EXACT": EXACT}
# marx.par defaults: ACIS_Exposure_Time + ACIS_Frame_Transfer_Time
ACIS_FRAME_TIME = 3.2 + 0.041


class EventParams(C.Structure):
    _fields_ = [("focal_length", C.c_double), ("det_offset", C.c_double * 3), ("roll_nom", C.c_double),
                ("frame_time", C.c_double), ("time_offset", C.c_double), ("dithered", C.c_int32),
                ("pixel_adjust", C.c_int32)]


class MxEvents(C.Structure):
    _fields_ = [("n", C.c_uint32), ("reserved", C.c_uint32), ("index", C.c_void_p),
                ("ccd_id", C.c_void_p), ("xpixel", C.c_void_p), ("ypixel", C.c_void_p),
                ("time", C.c_void_p), ("time64", C.c_void_p),
                ("sky_ra", C.c_void_p), ("sky_dec", C.c_void_p), ("sky_roll", C.c_void_p),
                ("det_dy", C.c_void_p), ("det_dz", C.c_void_p), ("det_theta", C.c_void_p),
                ("b_energy", C.c_void_p), ("uniforms", C.c_void_p),
                ("chipx", C.c_void_p), ("chipy", C.c_void_p),
                ("detx", C.c_void_p), ("dety", C.c_void_p), ("x", C.c_void_p), ("y", C.c_void_p),
                ("tdetx", C.c_void_p), ("tdety", C.c_void_p), ("expno", C.c_void_p),
                ("fltgrade", C.c_void_p), ("grade", C.c_void_p)]


# input columns: (struct field, numpy dtype)
INPUTS = {"index": ("index", np.uint32), "ccd": ("ccd_id", np.int8), "xpixel": ("xpixel", np.float32),
          "ypixel": ("ypixel", np.float32), "time": ("time", np.float32), "time64": ("time64", np.float64),
          "sky_ra": ("sky_ra", np.float32), "sky_dec": ("sky_dec", np.float32),
          "sky_roll": ("sky_roll", np.float32), "det_dy": ("det_dy", np.float32),
          "det_dz": ("det_dz", np.float32), "det_theta": ("det_theta", np.float32),
          "b_energy": ("b_energy", np.float32), "uniforms": ("uniforms", np.float64)}
OUTPUTS = {"chipx": np.float32, "chipy": np.float32, "detx": np.float64, "dety": np.float64, "x": np.float64,
           "y": np.float64, "tdetx": np.int32, "tdety": np.int32, "expno": np.int32, "fltgrade": np.int16,
           "grade": np.int16}


def params(focal_length=10070.0, det_offset=(0.0, 0.0, 0.0), roll_nom=0.0, frame_time=ACIS_FRAME_TIME,
           dithered=True, pixel_adjust=EDSER, time_offset=0.0) -> EventParams:
    p = EventParams()
    p.focal_length = focal_length
    p.det_offset[:] = list(det_offset)
    p.roll_nom = roll_nom
    p.frame_time = frame_time
    p.time_offset = time_offset
    p.dithered = 1 if dithered else 0
    p.pixel_adjust = PIXADJ[pixel_adjust] if isinstance(pixel_adjust, str) else int(pixel_adjust)
    return p


def _bind(L):
    if not getattr(L, "_mx_events_bound", False):
        L.mx_event_coords.argtypes = [C.c_void_p, C.POINTER(EventParams), C.POINTER(MxEvents), C.c_uint64,
                                      C.c_void_p]
        L.mx_event_coords_host.argtypes = [C.c_void_p, C.POINTER(EventParams), C.POINTER(MxEvents), C.c_uint64]
        L.mx_event_bad_count.argtypes = [C.c_void_p, C.POINTER(C.c_ulonglong), C.c_int]
        L._mx_events_bound = True
    return L


def event_coords_host(engine, p: EventParams, ev: dict, n: int | None = None, seed: int = 0) -> dict:
    """Host arrays in, host arrays out (every output column)."""
    L = _bind(engine.lib)
    n = len(ev["index"]) if ev.get("index") is not None else (n if n is not None else len(ev["ccd"]))
    s = MxEvents()
    s.n = n
    keep = []
    for k, (field, dt) in INPUTS.items():
        a = ev.get(k)
        if a is None:
            continue
        a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        setattr(s, field, a.ctypes.data)
    out = {k: np.zeros(n, dtype=dt) for k, dt in OUTPUTS.items()}
    for k, a in out.items():
        setattr(s, k, a.ctypes.data)
    engine._check(L.mx_event_coords_host(engine.h, C.byref(p), C.byref(s), seed))
    return out


def event_coords(engine, p: EventParams, ev: dict, n: int, seed: int = 0, stream=None) -> dict:
    """Device tensors in (dict of torch tensors, any of INPUTS), device
    tensors out; asynchronous on `stream` (default: torch's current)."""
    import torch
    L = _bind(engine.lib)
    dev = None
    s = MxEvents()
    s.n = n
    for k, (field, _) in INPUTS.items():
        t = ev.get(k)
        if t is None:
            continue
        assert t.is_cuda and t.is_contiguous(), k
        dev = t.device
        setattr(s, field, t.data_ptr())
    tmap = {np.float32: torch.float32, np.float64: torch.float64, np.int32: torch.int32, np.int16: torch.int16}
    out = {k: torch.empty(n, dtype=tmap[dt], device=dev) for k, dt in OUTPUTS.items()}
    for k, t in out.items():
        setattr(s, k, t.data_ptr())
    st = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    engine._check(L.mx_event_coords(engine.h, C.byref(p), C.byref(s), seed, C.c_void_p(st)))
    return out


def photon_events(ph, index) -> dict:
    """The event columns of a device photon list (``DevicePhotons``) for the
    photons `index` (device int32/uint32 tensor, e.g. Engine.compact):
    detector.dat, xpixel.dat, ypixel.dat, time and the dither state, as the
    writer would put them in an output directory."""
    s = ph.n
    return {"index": index, "ccd": ph.ccd_num, "xpixel": ph.y_pixel, "ypixel": ph.z_pixel,
            "time64": ph.arrival_time, "sky_ra": ph.dither_state[0], "sky_dec": ph.dither_state[1],
            "sky_roll": ph.dither_state[2]} if s else {}


def bad_count(engine, reset: bool = True) -> int:
    L = _bind(engine.lib)
    c = C.c_ulonglong(0)
    engine._check(L.mx_event_bad_count(engine.h, C.byref(c), 1 if reset else 0))
    return c.value
