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
GRATING = {"NONE": 0, "HETG": 1, "LETG": 2}
DETECTOR = {"NONE": 0, "ACIS-I": 1, "ACIS-S": 2, "HRC-I": 3, "HRC-S": 4}
# HRC blur parameter suffixes, in the order of mx_config.hrc_*_blur
HRC_BLUR = ("G1FWHM", "G1Xctr", "G1Yctr", "G1Amp", "G2FWHM", "G2Xctr", "G2Yctr", "G2Amp",
            "L1FWHM", "L1Xctr", "L1Yctr", "L1Amp", "L1Rmax")
DITHER = {"NONE": 0, "INTERNAL": 1, "FILE": 2}


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
        ("letg_theta", C.c_double * 4), ("letg_dtheta", C.c_double * 4),
        ("letg_period", C.c_double * 4), ("letg_dpp", C.c_double * 4), ("letg_vig", C.c_double * 4),
        ("leg_rowland", C.c_double), ("letg_acis_dtheta", C.c_double),
        ("leg_fine_orders", C.c_int32), ("leg_coarse_orders", C.c_int32),
        ("leg_fine_period", C.c_double), ("leg_fine_bar_height", C.c_double), ("leg_fine_bar_width", C.c_double),
        ("leg_coarse_period", C.c_double), ("leg_coarse_bar_height", C.c_double),
        ("leg_coarse_bar_width", C.c_double),
        ("det_ideal", C.c_int32), ("reserved2", C.c_int32),
        ("hrc_i_blur", C.c_double * 13), ("hrc_s_blur", C.c_double * 13),
        ("hrc_hesf", C.c_int32), ("hesf_n", C.c_int32),
        ("hesf_offset_x", C.c_double), ("hesf_offset_z", C.c_double),
        ("hesf_gap_y1", C.c_double), ("hesf_gap_y2", C.c_double),
        ("hesf_length", C.c_double), ("hesf_cr_width", C.c_double),
        ("hesf_height", C.c_double * 4), ("hesf_theta", C.c_double * 4),
        ("ra_nom", C.c_double), ("dec_nom", C.c_double), ("pointing_offset", C.c_double * 2),
        ("tstart_mjdsecs", C.c_double),
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
    c.letg_theta[:] = [0.07] * 4
    c.letg_dtheta[:] = [0.617] * 4
    c.letg_period[:] = [0.991216] * 4
    c.letg_dpp[:] = [78e-6] * 4
    c.letg_vig[:] = [1.0] * 4
    c.leg_rowland = 8637.0
    c.letg_acis_dtheta = -0.0867
    c.leg_fine_orders, c.leg_coarse_orders = 19, 121
    c.leg_fine_period, c.leg_fine_bar_height, c.leg_fine_bar_width = 25.4, 2.5, 2.5
    c.leg_coarse_period, c.leg_coarse_bar_height, c.leg_coarse_bar_width = 2000.0, 26.0, 68.0
    c.det_ideal = 0
    c.hrc_i_blur[:] = [13.8994, 64.1124, 64.5285, 15.7528, 4.25636, 61.35, 64.178, 0.0,
                       10.8269, 73.3361, 63.9927, 0.0, 256.0]
    c.hrc_s_blur[:] = [13.900, 64.110, 64.530, 15.750, 4.2560, 67.420, 64.110, 0.0,
                       10.820, 53.030, 63.880, 0.0, 256.000]
    c.hrc_hesf, c.hesf_n = 1, 2
    c.hesf_offset_x, c.hesf_offset_z = 26.3, -5.359
    c.hesf_gap_y1, c.hesf_gap_y2 = 28.7, 36.7
    c.hesf_length, c.hesf_cr_width = 294.0, 15.7
    c.hesf_height[:] = [22.3, 50.0, 0.0, 0.0]
    c.hesf_theta[:] = [4.5, 7.0, 0.0, 0.0]
    c.ra_nom, c.dec_nom = 250.2134679741175, -53.75743813458669
    c.pointing_offset[:] = [0.0, 0.0]
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
        "LEGRowlandDiameter": repr(c.leg_rowland), "LETG_ACIS_dTheta": repr(c.letg_acis_dtheta),
        "legFineNumOrders": str(c.leg_fine_orders), "legCoarseNumOrders": str(c.leg_coarse_orders),
        "legFinePeriod": repr(c.leg_fine_period), "legFineBarHeight": repr(c.leg_fine_bar_height),
        "legFineBarWidth": repr(c.leg_fine_bar_width), "legCoarsePeriod": repr(c.leg_coarse_period),
        "legCoarseBarHeight": repr(c.leg_coarse_bar_height), "legCoarseBarWidth": repr(c.leg_coarse_bar_width),
        "DetIdeal": _yn(c.det_ideal),
    }
    for k, name in enumerate(HRC_BLUR):
        P[f"HRC-I-Blur{name}"] = repr(c.hrc_i_blur[k])
        P[f"HRC-S-Blur{name}"] = repr(c.hrc_s_blur[k])
    P["RA_Nom"], P["Dec_Nom"] = repr(c.ra_nom), repr(c.dec_nom)
    P["PointingOffsetY"], P["PointingOffsetZ"] = repr(c.pointing_offset[0]), repr(c.pointing_offset[1])
    P["HRC-HESF"] = _yn(c.hrc_hesf)
    P["HESFN"] = str(c.hesf_n)
    P["HESFOffsetX"], P["HESFOffsetZ"] = repr(c.hesf_offset_x), repr(c.hesf_offset_z)
    P["HESFGapY1"], P["HESFGapY2"] = repr(c.hesf_gap_y1), repr(c.hesf_gap_y2)
    P["HESFLength"], P["HESFCrWidth"] = repr(c.hesf_length), repr(c.hesf_cr_width)
    for k in range(4):
        P[f"HESFHeight{k + 1}"] = repr(c.hesf_height[k])
        P[f"HESFTheta{k + 1}"] = repr(c.hesf_theta[k])
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
        P[f"LETG_Shell{s}_Theta"] = repr(c.letg_theta[i])
        P[f"LETG_Shell{s}_dTheta"] = repr(c.letg_dtheta[i])
        P[f"LETG_Shell{s}_Period"] = repr(c.letg_period[i])
        P[f"LETG_Shell{s}_dPoverP"] = repr(c.letg_dpp[i])
        P[f"LETG_Shell{s}_Vig"] = repr(c.letg_vig[i])
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
        c.letg_theta[i] = num(f"LETG_Shell{s}_Theta", c.letg_theta[i])
        c.letg_dtheta[i] = num(f"LETG_Shell{s}_dTheta", c.letg_dtheta[i])
        c.letg_period[i] = num(f"LETG_Shell{s}_Period", c.letg_period[i])
        c.letg_dpp[i] = num(f"LETG_Shell{s}_dPoverP", c.letg_dpp[i])
        c.letg_vig[i] = num(f"LETG_Shell{s}_Vig", c.letg_vig[i])
    c.leg_rowland = num("LEGRowlandDiameter", c.leg_rowland)
    c.letg_acis_dtheta = num("LETG_ACIS_dTheta", c.letg_acis_dtheta)
    c.leg_fine_orders = int(num("legFineNumOrders", c.leg_fine_orders))
    c.leg_coarse_orders = int(num("legCoarseNumOrders", c.leg_coarse_orders))
    for k in ("period", "bar_height", "bar_width"):
        name = "".join(w.capitalize() for w in k.split("_"))
        setattr(c, f"leg_fine_{k}", num(f"legFine{name}", getattr(c, f"leg_fine_{k}")))
        setattr(c, f"leg_coarse_{k}", num(f"legCoarse{name}", getattr(c, f"leg_coarse_{k}")))
    c.det_ideal = yes("DetIdeal", c.det_ideal)
    for k, name in enumerate(HRC_BLUR):
        c.hrc_i_blur[k] = num(f"HRC-I-Blur{name}", c.hrc_i_blur[k])
        c.hrc_s_blur[k] = num(f"HRC-S-Blur{name}", c.hrc_s_blur[k])
    c.ra_nom, c.dec_nom = num("RA_Nom", c.ra_nom), num("Dec_Nom", c.dec_nom)
    c.pointing_offset[0] = num("PointingOffsetY", c.pointing_offset[0])
    c.pointing_offset[1] = num("PointingOffsetZ", c.pointing_offset[1])
    c.hrc_hesf = yes("HRC-HESF", c.hrc_hesf)
    c.hesf_n = int(num("HESFN", c.hesf_n))
    c.hesf_offset_x, c.hesf_offset_z = num("HESFOffsetX", c.hesf_offset_x), num("HESFOffsetZ", c.hesf_offset_z)
    c.hesf_gap_y1, c.hesf_gap_y2 = num("HESFGapY1", c.hesf_gap_y1), num("HESFGapY2", c.hesf_gap_y2)
    c.hesf_length, c.hesf_cr_width = num("HESFLength", c.hesf_length), num("HESFCrWidth", c.hesf_cr_width)
    for k in range(4):
        c.hesf_height[k] = num(f"HESFHeight{k + 1}", c.hesf_height[k])
        c.hesf_theta[k] = num(f"HESFTheta{k + 1}", c.hesf_theta[k])
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
