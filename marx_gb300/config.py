"""Simulation parameters: the ``mx_config`` struct of include/marx_gb300.h.

Field names follow the MARX parameter file (marx/par/marx.par); the
defaults are that file's values.  ``to_par`` renders a config as the
``Name=value`` overrides MARX itself accepts, and ``from_par`` reads a MARX
``.par`` file into a config, so a user's existing parameter file drives the
engine unchanged.
"""
from __future__ import annotations

import ctypes as C

SHELLS = (1, 3, 4, 6)
GRATING = {"NONE": 0, "HETG": 1}
DETECTOR = {"NONE": 0, "ACIS-I": 1, "ACIS-S": 2}
DITHER = {"NONE": 0, "INTERNAL": 1}


class MxConfig(C.Structure):
    _fields_ = [
        ("hrma_cap_x", C.c_double),
        ("shell_xoffset", C.c_double * 4),
        ("blur_p", C.c_double * 4), ("blur_h", C.c_double * 4),
        ("scat_p", C.c_double * 4), ("scat_h", C.c_double * 4),
        ("hrma_vig", C.c_double),
        ("hrma_ideal", C.c_int32), ("use_blur", C.c_int32), ("use_wfold", C.c_int32),
        ("use_struts", C.c_int32), ("use_scale_factors", C.c_int32),
        ("shutters", C.c_uint32 * 4),
        ("source_distance", C.c_double),
        ("grating", C.c_int32), ("use_sector_files", C.c_int32),
        ("hetg_theta", C.c_double * 4), ("hetg_dtheta", C.c_double * 4),
        ("hetg_period", C.c_double * 4), ("hetg_dpp", C.c_double * 4),
        ("hetg_vig", C.c_double * 4),
        ("meg_rowland", C.c_double), ("heg_rowland", C.c_double),
        ("max_order", C.c_int32), ("aperture_area_uniform", C.c_int32),
        ("dither", C.c_int32), ("reserved1", C.c_int32),
        ("dither_amp", C.c_double * 3), ("dither_period", C.c_double * 3),
        ("dither_phase", C.c_double * 3),
        ("roll_nom", C.c_double), ("aspect_blur", C.c_double),
        ("detector", C.c_int32), ("det_extend", C.c_int32),
        ("det_offset", C.c_double * 3),
        ("acis_exposure_time", C.c_double), ("acis_frame_transfer_time", C.c_double),
        ("focal_length", C.c_double),
        ("start_time", C.c_double),
    ]


def default_config() -> MxConfig:
    """marx.par (MARX 5.5) defaults for every field."""
    c = MxConfig()
    c.hrma_cap_x = 10079.771554
    c.shell_xoffset[:] = [-3.277664, -0.257891, 0.733315, -0.541755]
    c.blur_p[:] = [0.303427, 0.0951899, 0.178899, 0.151085]
    c.blur_h[:] = [0.0051428, 0.0713614, 0.0101367, 0.0239287]
    c.scat_p[:] = [2.8420331, 1.7305226, 1.0077613, 2.1199425]
    c.scat_h[:] = [3.2451338, 2.4618956, 2.9027099, 2.0209803]
    c.hrma_vig = 1.0
    c.hrma_ideal, c.use_blur, c.use_wfold, c.use_struts, c.use_scale_factors = 0, 1, 1, 1, 1
    c.shutters[:] = [0xF] * 4
    c.source_distance = 0.0
    c.grating, c.use_sector_files = GRATING["HETG"], 1
    c.hetg_theta[:] = [4.755, 4.755, -5.205, -5.205]
    c.hetg_dtheta[:] = [1.5] * 4
    c.hetg_period[:] = [0.400195, 0.400195, 0.200081, 0.200081]
    c.hetg_dpp[:] = [162e-6, 162e-6, 146e-6, 146e-6]
    c.hetg_vig[:] = [1.0] * 4
    c.meg_rowland = c.heg_rowland = 8632.48
    c.max_order = 0
    c.aperture_area_uniform = 0
    c.dither = DITHER["INTERNAL"]
    c.dither_amp[:] = [16.0, 16.0, 0.0]
    c.dither_period[:] = [1414.2, 2000.0, 1e5]
    c.dither_phase[:] = [0.0, 0.0, 0.0]
    c.roll_nom = 237.36968458476
    c.aspect_blur = 0.07
    c.detector, c.det_extend = DETECTOR["ACIS-S"], 0
    c.det_offset[:] = [0.0, 0.0, 0.0]
    c.acis_exposure_time, c.acis_frame_transfer_time = 3.2, 0.041
    c.focal_length = 10065.5
    c.start_time = 0.0
    return c


def copy_config(c: MxConfig) -> MxConfig:
    d = MxConfig()
    C.pointer(d)[0] = c
    return d


def _yn(v) -> str:
    return "yes" if v else "no"


def _shutter_string(bitmap: int) -> str:
    # _marx_parse_shutter_string (mirror.c:112): '0' = open sets bit q
    return "".join("0" if bitmap & (1 << q) else "1" for q in range(4))


def to_par(c: MxConfig) -> dict:
    """The MARX parameter overrides equivalent to ``c``."""
    inv = lambda d, v: {b: a for a, b in d.items()}[v]
    P = {
        "MirrorType": "HRMA",
        "HRMA_Cap_X": repr(c.hrma_cap_x), "HRMAVig": repr(c.hrma_vig),
        "HRMA_Ideal": _yn(c.hrma_ideal), "HRMA_Use_Blur": _yn(c.use_blur),
        "HRMA_Use_WFold": _yn(c.use_wfold), "HRMA_Use_Struts": _yn(c.use_struts),
        "HRMA_Use_Scale_Factors": _yn(c.use_scale_factors),
        "GratingType": inv(GRATING, c.grating),
        "Use_HETG_Sector_Files": _yn(c.use_sector_files),
        "UseGratingEffFiles": "yes",
        "MEGRowlandDiameter": repr(c.meg_rowland), "HEGRowlandDiameter": repr(c.heg_rowland),
        "DitherModel": inv(DITHER, c.dither),
        "Roll_Nom": repr(c.roll_nom), "AspectBlur": repr(c.aspect_blur),
        "DetectorType": inv(DETECTOR, c.detector), "DetExtendFlag": _yn(c.det_extend),
        "DetOffsetX": repr(c.det_offset[0]), "DetOffsetY": repr(c.det_offset[1]),
        "DetOffsetZ": repr(c.det_offset[2]),
        "ACIS_Exposure_Time": repr(c.acis_exposure_time),
        "ACIS_Frame_Transfer_Time": repr(c.acis_frame_transfer_time),
        "Verbose": "0",
    }
    for i, s in enumerate(SHELLS):
        P[f"HRMA_P{s}H{s}_XOffset"] = repr(c.shell_xoffset[i])
        P[f"P{s}Blur"], P[f"H{s}Blur"] = repr(c.blur_p[i]), repr(c.blur_h[i])
        P[f"P{s}ScatFactor"], P[f"H{s}ScatFactor"] = repr(c.scat_p[i]), repr(c.scat_h[i])
        P[f"Shutters{s}"] = _shutter_string(c.shutters[i])
        P[f"HETG_Shell{s}_Theta"] = repr(c.hetg_theta[i])
        P[f"HETG_Shell{s}_dTheta"] = repr(c.hetg_dtheta[i])
        P[f"HETG_Shell{s}_Period"] = repr(c.hetg_period[i])
        P[f"HETG_Shell{s}_dPoverP"] = repr(c.hetg_dpp[i])
        P[f"HETG_Shell{s}_Vig"] = repr(c.hetg_vig[i])
    for k, ax in enumerate(("RA", "Dec", "Roll")):
        P[f"DitherAmp_{ax}"] = repr(c.dither_amp[k])
        P[f"DitherPeriod_{ax}"] = repr(c.dither_period[k])
        P[f"DitherPhase_{ax}"] = repr(c.dither_phase[k])
    return P


def from_par(path: str, overrides: dict | None = None) -> MxConfig:
    """Read a MARX .par file (name,type,mode,value,...) into a config."""
    vals = {}
    for line in open(path):
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        f = next(__import__("csv").reader([line]))
        if len(f) >= 4:
            vals[f[0]] = f[3]
    vals.update(overrides or {})
    c = default_config()
    num = lambda k, d: float(vals[k]) if k in vals else d
    yes = lambda k, d: (vals[k].strip().lower() in ("yes", "y", "true", "1")) if k in vals else d
    c.hrma_cap_x = num("HRMA_Cap_X", c.hrma_cap_x)
    c.hrma_vig = num("HRMAVig", c.hrma_vig)
    c.hrma_ideal = yes("HRMA_Ideal", c.hrma_ideal)
    c.use_blur = yes("HRMA_Use_Blur", c.use_blur)
    c.use_wfold = yes("HRMA_Use_WFold", c.use_wfold)
    c.use_struts = yes("HRMA_Use_Struts", c.use_struts)
    c.use_scale_factors = yes("HRMA_Use_Scale_Factors", c.use_scale_factors)
    for i, s in enumerate(SHELLS):
        c.shell_xoffset[i] = num(f"HRMA_P{s}H{s}_XOffset", c.shell_xoffset[i])
        c.blur_p[i] = num(f"P{s}Blur", c.blur_p[i]); c.blur_h[i] = num(f"H{s}Blur", c.blur_h[i])
        c.scat_p[i] = num(f"P{s}ScatFactor", c.scat_p[i]); c.scat_h[i] = num(f"H{s}ScatFactor", c.scat_h[i])
        if f"Shutters{s}" in vals:
            c.shutters[i] = sum(1 << q for q, ch in enumerate(vals[f"Shutters{s}"]) if ch == "0")
        c.hetg_theta[i] = num(f"HETG_Shell{s}_Theta", c.hetg_theta[i])
        c.hetg_dtheta[i] = num(f"HETG_Shell{s}_dTheta", c.hetg_dtheta[i])
        c.hetg_period[i] = num(f"HETG_Shell{s}_Period", c.hetg_period[i])
        c.hetg_dpp[i] = num(f"HETG_Shell{s}_dPoverP", c.hetg_dpp[i])
        c.hetg_vig[i] = num(f"HETG_Shell{s}_Vig", c.hetg_vig[i])
    if "GratingType" in vals:
        c.grating = GRATING[vals["GratingType"]]
    c.use_sector_files = yes("Use_HETG_Sector_Files", c.use_sector_files)
    c.meg_rowland = num("MEGRowlandDiameter", c.meg_rowland)
    c.heg_rowland = num("HEGRowlandDiameter", c.heg_rowland)
    if "DitherModel" in vals:
        c.dither = DITHER[vals["DitherModel"]]
    for k, ax in enumerate(("RA", "Dec", "Roll")):
        c.dither_amp[k] = num(f"DitherAmp_{ax}", c.dither_amp[k])
        c.dither_period[k] = num(f"DitherPeriod_{ax}", c.dither_period[k])
        c.dither_phase[k] = num(f"DitherPhase_{ax}", c.dither_phase[k])
    c.roll_nom = num("Roll_Nom", c.roll_nom)
    c.aspect_blur = num("AspectBlur", c.aspect_blur)
    if "DetectorType" in vals:
        c.detector = DETECTOR[vals["DetectorType"]]
    c.det_extend = yes("DetExtendFlag", c.det_extend)
    for k, ax in enumerate("XYZ"):
        c.det_offset[k] = num(f"DetOffset{ax}", c.det_offset[k])
    c.acis_exposure_time = num("ACIS_Exposure_Time", c.acis_exposure_time)
    c.acis_frame_transfer_time = num("ACIS_Frame_Transfer_Time", c.acis_frame_transfer_time)
    return c
