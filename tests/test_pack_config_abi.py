"""Host-side pieces that need no GPU: the table pack, parameter handling,
configuration validation, and the C ABI library's exports."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from marx_gb300 import config as cfgmod
from marx_gb300.caldb.pack import DEFAULT_PACK, read_pack, write_pack
from marx_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_pack_holds_every_table():
    S = read_pack(DEFAULT_PACK)
    assert S["hrma/rdb"].shape == (8, 9)
    assert S["hrma/optconst"].shape[0] == 3
    for s in (1, 3, 4, 6):
        assert S[f"hrma/corr{s}"].shape[0] == 2
        for k in "ph":
            h = S[f"wfold/{k}{s}/hdr"]
            assert np.all(np.diff(h[:, 0]) > 0)           # sorted by E sin(alpha), no duplicates
            assert S[f"wfold/{k}{s}/theta"].shape[0] == h.shape[0]
    for i in range(4):
        e = S[f"hetg/geff{i}/energy"]
        assert np.all(np.diff(e) >= 0)
        assert S[f"hetg/geff{i}/eff"].shape == (23, e.size)
    assert S["acis/geom"].shape == (10, 13)


def test_pack_round_trip(tmp_path):
    S = {"a": np.arange(5, dtype=np.float64), "b/c": np.ones((2, 3), np.float32), "d": np.array([7], np.int32)}
    p = tmp_path / "t.mxpack"
    write_pack(str(p), S)
    T = read_pack(str(p))
    for k in S:
        assert T[k].dtype == S[k].dtype and np.array_equal(T[k], S[k])


def test_par_round_trip(tmp_path):
    c = W.plain_scatter().cfg
    par = cfgmod.to_par(c)
    lines = [f'{k},s,h,"{v}",,,""' for k, v in par.items()]
    p = tmp_path / "x.par"
    p.write_text("\n".join(lines) + "\n")
    d = cfgmod.from_par(str(p))
    assert bytes(d) == bytes(c)


def _native():
    from marx_gb300.build import build
    build()
    from marx_gb300 import _native
    return _native


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "marx_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mx_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_function():
    L = _native().load_library()
    names = declared_functions()
    assert len(names) >= 14
    for n in names:
        assert hasattr(L, n), n


def test_validate_config_rejects_bad_values():
    nat = _native()
    c = cfgmod.default_config()
    assert nat.validate_config(c) is None
    bad = cfgmod.copy_config(c); bad.hrma_vig = 1.5
    assert "HRMAVig" in nat.validate_config(bad)
    bad = cfgmod.copy_config(c); bad.shutters[:] = [0, 0, 0, 0]
    assert "area is 0" in nat.validate_config(bad)
    bad = cfgmod.copy_config(c); bad.acis_exposure_time = 0
    assert "Exposure" in nat.validate_config(bad)
    bad = cfgmod.copy_config(c); bad.detector = 7
    assert nat.validate_config(bad) is not None
    assert nat.validate_config(c, pack="/nonexistent.mxpack") is not None


def test_engine_fails_loudly_without_a_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    nat = _native()
    with pytest.raises(RuntimeError):
        nat.Engine(cfgmod.default_config())


def test_default_config_matches_c_defaults():
    L = _native().load_library()
    c = cfgmod.MxConfig()
    L.mx_config_default(C.byref(c))
    assert bytes(c) == bytes(cfgmod.default_config())


def _source_direction(cfg, ra, dec):
    import ctypes as C
    from marx_gb300.config import MxConfig
    L = _native().load_library()
    L.mx_source_direction.argtypes = [C.POINTER(MxConfig), C.c_double, C.c_double, C.POINTER(C.c_double)]
    out = (C.c_double * 3)()
    r = L.mx_source_direction(C.byref(cfg), ra, dec, out)
    return r, np.array(out[:])


def test_source_direction_matches_reference_fixture():
    """The source direction st->p the reference computed from SourceRA/Dec
    and the pointing (tests/golden/sources.npz)."""
    import os
    from marx_gb300 import workloads as W
    from helpers import GOLDEN
    z = np.load(os.path.join(GOLDEN, "sources.npz"))
    cfg = W.plain_onaxis(parity=True).cfg
    r, p = _source_direction(cfg, 250.25, -53.73)
    assert r == 0
    assert np.abs(p - z["point_src"]).max() <= 1e-15, (p, z["point_src"])


def test_source_direction_matches_reference_live():
    import pytest
    from oracle.bindings import Reference, reference_available
    from marx_gb300 import workloads as W
    from marx_gb300.config import DITHER
    if not reference_available():
        pytest.skip("reference sources not present")
    cases = [(250.20, -53.70, 0.0, 0.0, 0.0), (250.31, -53.80, 237.36968458476, 3.0, -2.0),
             (250.2134679741175, -53.75743813458669, 90.0, 0.0, 0.0)]
    for ra, dec, roll, oy, oz in cases:
        for dither in ("NONE", "INTERNAL"):
            cfg = W.plain_onaxis(parity=True).cfg
            cfg.roll_nom = roll
            cfg.pointing_offset[:] = [oy, oz]
            cfg.dither = DITHER[dither]
            ref = Reference(cfg, extra_par={"SourceRA": repr(ra), "SourceDEC": repr(dec)})
            p_ref, _, _ = ref.source_photons(1, np.full((4, 1), 0.5))
            r, p = _source_direction(cfg, ra, dec)
            assert r == 0 and np.abs(p - p_ref).max() <= 1e-15, (ra, dec, roll, dither, p, p_ref)


def _read_par_c(L, path, overrides=()):
    L.mx_config_read_par.argtypes = [C.POINTER(cfgmod.MxConfig), C.c_char_p, C.POINTER(C.c_char_p), C.c_int]
    c = cfgmod.MxConfig()
    arr = (C.c_char_p * max(1, len(overrides)))(*[o.encode() for o in overrides])
    rc = L.mx_config_read_par(C.byref(c), path.encode(), arr, len(overrides))
    return rc, c


@pytest.mark.parametrize("name", list(W.ALL))
def test_c_par_reader_matches_python_reader(tmp_path, name):
    """mx_config_read_par (the C ABI's parameter-file reader) gives the same
    configuration as from_par on a parameter file of every workload, with
    the marx.par type letter of each parameter."""
    L = _native().load_library()
    L.mx_param_type.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_uint32)]
    c = W.ALL[name]().cfg
    lines = []
    for k, v in cfgmod.to_par(c).items():
        t = C.create_string_buffer(1)
        if L.mx_param_type(k.encode(), t, None) != 0:
            continue            # read by no engine module (Verbose, UseGratingEffFiles)
        lines.append(f'{k},{t.value.decode()},h,"{v}",,,""')
    p = tmp_path / "w.par"
    p.write_text("\n".join(lines) + "\n")
    rc, d = _read_par_c(L, str(p))
    assert rc == 0, L.mx_last_error(None)
    e = cfgmod.from_par(str(p))
    for f, _ in cfgmod.MxConfig._fields_:
        if f in ("max_order", "aperture_area_uniform", "source_distance", "start_time", "focal_length",
                 "tstart_mjdsecs"):
            continue            # engine settings, not marx.par parameters
        val = lambda o: getattr(o, f)[:] if hasattr(getattr(o, f), "_length_") else getattr(o, f)  # noqa: E731
        assert repr(val(d)) == repr(val(e)), f


def test_c_par_reader_overrides_and_errors(tmp_path):
    L = _native().load_library()
    p = tmp_path / "o.par"
    p.write_text('GratingType,s,h,"HETG",,,""\nHRMA_Use_Blur,b,h,yes,,,""\nShutters3,s,h,"0101",,,""\n')
    rc, c = _read_par_c(L, str(p), ["GratingType=LETG", "DetectorType=HRC-S", "P3Blur=0.25"])
    assert rc == 0
    assert c.grating == cfgmod.GRATING["LETG"] and c.detector == cfgmod.DETECTOR["HRC-S"]
    assert c.use_blur == 1 and c.shutters[1] == 0b0101 and c.blur_p[1] == 0.25
    for bad in (["GratingType=XTG"], ["HRMA_Use_Blur=maybe"], ["Shutters1=01"], ["P1Blur=abc"], ["MirrorType=FLATFIELD"],
                ["DitherModel"]):
        rc, _ = _read_par_c(L, str(p), bad)
        assert rc == -1, bad


def test_c_par_reader_reads_the_reference_parameter_file():
    from oracle.bindings import REF_ROOT, reference_available
    if not reference_available():
        pytest.skip("the reference checkout is not on this machine")
    path = os.path.join(REF_ROOT, "marx", "par", "marx.par")
    L = _native().load_library()
    rc, d = _read_par_c(L, path)
    assert rc == 0, L.mx_last_error(None)
    assert bytes(d) == bytes(cfgmod.from_par(path))
