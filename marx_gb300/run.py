"""marx's main loop on the GPU (mx_run_marx in include/marx_gb300.h).

    write_par("sim.par", cfg, NumRays=100000, SourceType="POINT", ...)
    stats = run_marx("sim.par", ["OutputDir=out", "RandomSeed=3"])

``write_par`` renders a configuration and run parameters as a MARX
parameter file (name,type,mode,value,min,max,prompt per line); the run reads
it as the marx program reads marx.par, overrides as on its command line.
"""
from __future__ import annotations

import ctypes as C

from .config import MxConfig, to_par

# the run parameters the loop reads besides the engine's (marx.c:789-805,
# source.c:77-88, spectrum.c:118-274, s-*.c) and their marx.par types
RUN_PARAMS = {
    "NumRays": "i", "dNumRays": "i", "ExposureTime": "r", "OutputDir": "f", "OutputVectors": "s",
    "RandomSeed": "i", "DumpToRayFile": "b", "RayFile": "f", "SourceType": "s", "SourceRA": "r", "SourceDEC": "r",
    "SourceDistance": "r", "SourceFlux": "r", "SpectrumType": "s", "SpectrumFile": "f", "MinEnergy": "r",
    "MaxEnergy": "r", "S-GaussSigma": "r", "S-BetaCoreRadius": "r", "S-BetaBeta": "r", "S-DiskTheta0": "r",
    "S-DiskTheta1": "r", "S-LinePhi": "r", "S-LineTheta": "r", "MirrorType": "s", "Verbose": "i",
}
RUN_DEFAULTS = {
    "NumRays": 100000, "dNumRays": 100000, "ExposureTime": 0.0, "OutputDir": "point", "RandomSeed": -1,
    "OutputVectors": "ETXYZ123DxyMPOabcdSrB", "DumpToRayFile": "no", "RayFile": "marx.rays", "SourceType": "POINT",
    "SourceRA": 250.2134679741175, "SourceDEC": -53.75743813458669, "SourceDistance": 0.0, "SourceFlux": 0.02,
    "SpectrumType": "FLAT", "SpectrumFile": "none", "MinEnergy": 1.775, "MaxEnergy": 1.775, "S-GaussSigma": 0.5,
    "S-BetaCoreRadius": 0.5, "S-BetaBeta": 0.5, "S-DiskTheta0": 0.0, "S-DiskTheta1": 20.0, "S-LinePhi": 0.0,
    "S-LineTheta": 30.0, "MirrorType": "HRMA", "Verbose": 0,
}


class MxRunStats(C.Structure):
    _fields_ = [("collected", C.c_uint64), ("detected", C.c_uint64), ("total_time", C.c_double),
                ("iterations", C.c_uint32), ("reserved", C.c_uint32)]


def _lib():
    from ._native import load_library
    L = load_library()
    if not getattr(L, "_mx_run_bound", False):
        L.mx_run_marx.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_char_p), C.c_int, C.POINTER(MxRunStats)]
        L.mx_param_type.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_uint32)]
        L._mx_run_bound = True
    return L


def write_par(path: str, cfg: MxConfig, **run) -> None:
    """A MARX parameter file: the marx.par MARX ships (kept in the table
    pack) with cfg's parameters and the run's (the defaults above, updated by
    the keyword arguments) set, so that every program reading it (marx2fits
    too) finds all of its parameters."""
    from .caldb.pack import DEFAULT_PACK, read_pack, section_text
    from .output import _par_lines, _par_set
    L = _lib()
    vals = dict(RUN_DEFAULTS)
    vals.update(run)
    lines = _par_lines(section_text(read_pack(DEFAULT_PACK)["par/marx"]).decode())
    for k, v in to_par(cfg).items():
        t = C.create_string_buffer(1)
        if L.mx_param_type(k.encode(), t, None) == 0:
            _par_set(lines, k, v, t.value.decode())
    for k, v in vals.items():
        t = RUN_PARAMS[k]
        _par_set(lines, k, ("yes" if v else "no") if isinstance(v, bool) else v, t)
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def geometric_area(cfg: MxConfig, pack: str | None = None) -> float:
    """The mirror's open aperture area in cm^2 (mx_geometric_area)."""
    from .caldb.pack import DEFAULT_PACK
    L = _lib()
    L.mx_geometric_area.argtypes = [C.c_char_p, C.POINTER(MxConfig), C.POINTER(C.c_double)]
    a = C.c_double(0.0)
    if L.mx_geometric_area((pack or DEFAULT_PACK).encode(), C.byref(cfg), C.byref(a)) != 0:
        raise RuntimeError("mx_geometric_area: " + L.mx_last_error(None).decode())
    return a.value


def run_marx(par_path: str, overrides=(), pack: str | None = None) -> dict:
    """Run the main loop; returns the run's counts and exposure."""
    from .caldb.pack import DEFAULT_PACK
    L = _lib()
    ov = [o.encode() for o in overrides]
    arr = (C.c_char_p * max(1, len(ov)))(*ov)
    st = MxRunStats()
    r = L.mx_run_marx((pack or DEFAULT_PACK).encode(), par_path.encode(), arr, len(ov), C.byref(st))
    if r != 0:
        raise RuntimeError(f"mx_run_marx: error {r}: " + L.mx_last_error(None).decode())
    return {"collected": st.collected, "detected": st.detected, "total_time": st.total_time,
            "iterations": st.iterations}
