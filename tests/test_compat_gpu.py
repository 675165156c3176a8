"""The compatibility shim on the GPU: a C driver (tests/compat/stage_fixture.c)
compiled against include/marx_gb300_compat.h and linked with
libmarx_gb300_compat.so runs MARX's stage calls (dither, then
marx_mirror_reflect, marx_grating_diffract, marx_detect, marx_prune_photons)
over a Marx_Photon_Type built from a reference fixture's photons and
pre-drawn variates, its parameters read through pf_get_* by name.  Every
attribute is compared with what the compiled reference wrote for the same
photons, under the parity contract; history bits, the skip of a stage that
already ran and the final prune are checked too."""
import os
import subprocess

import numpy as np
import pytest

from marx_gb300 import config as cfgmod
from marx_gb300 import workloads as W

from helpers import load_trace_fixture, X_TOL_MM, P_TOL, EXTRA_FIELDS
from test_compat import ATTR_DTYPE

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HIST = {"energy": 0x1, "time": 0x2, "x": 0x4, "p": 0x8, "tag": 0x10, "pha": 0x20, "pi": 0x40, "pixel": 0x80,
        "num": 0x100, "region": 0x200, "uv": 0x400, "shell": 0x800, "order": 0x100000, "o1": 0x200000,
        "o2": 0x400000, "o3": 0x800000, "o4": 0x1000000}


@pytest.fixture(scope="module")
def driver(cuda, tmp_path_factory):
    from marx_gb300.build import OUT
    exe = tmp_path_factory.mktemp("compat") / "stage_fixture"
    # -rdynamic: the driver's pf_get_* are what the shim's weak references bind to
    subprocess.run(["gcc", "-O2", "-rdynamic", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "compat", "stage_fixture.c"), "-o", str(exe),
                    "-L", OUT, "-lmarx_gb300_compat", f"-Wl,-rpath,{OUT}"], check=True)
    return str(exe)


def _params(cfg, path):
    from marx_gb300._native import load_library
    import ctypes as C
    L = load_library()
    L.mx_param_type.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_uint32)]
    lines = ["RandomSeed=0"]
    for k, v in cfgmod.to_par(cfg).items():
        if L.mx_param_type(k.encode(), None, None) == 0:
            lines.append(f"{k}={v}")
    open(path, "w").write("\n".join(lines) + "\n")


def _run(driver, tmp_path, w, ph, U, N):
    n = ph.n
    _params(w.cfg, tmp_path / "p.txt")
    with open(tmp_path / "in.bin", "wb") as f:
        f.write(np.uint32(n).tobytes())
        for a in (ph.energy, ph.p, ph.arrival_time):
            f.write(np.ascontiguousarray(a, np.float64).tobytes())
        f.write(np.ascontiguousarray(ph.tag, np.uint32).tobytes())
        f.write(np.ascontiguousarray(U[:36], np.float64).tobytes())
        f.write(np.ascontiguousarray(N[:24], np.float64).tobytes())
    r = subprocess.run([driver, str(tmp_path / "p.txt"), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stderr)
    b = open(tmp_path / "out.bin", "rb").read()
    rc = np.frombuffer(b[:16], np.int32)
    hist = int(np.frombuffer(b[16:24], np.uint64)[0])
    m = int(np.frombuffer(b[24:28], np.uint32)[0])
    idx = np.frombuffer(b[28:28 + 4 * m], np.uint32)
    o = 28 + 4 * m
    same = int(np.frombuffer(b[o:o + 4], np.int32)[0])
    attrs = np.frombuffer(b[o + 4:], ATTR_DTYPE)
    assert attrs.size == n
    return rc, hist, idx, same, attrs


@pytest.mark.parametrize("name", list(W.ALL))
def test_shim_matches_reference_fixture(driver, tmp_path, name):
    w, ph, U, N, z = load_trace_fixture(name)
    rc, hist, idx, same, a = _run(driver, tmp_path, w, ph, U, N)
    cfg = w.cfg
    det_id = {0: 0, 1: 4, 2: 3, 3: 2, 4: 1}[cfg.detector]
    assert list(rc) == [0, 2, cfg.grating, det_id]
    # attributes against the reference's own trace of the same photons
    assert np.abs(a["x"].T - z["x"]).max() <= X_TOL_MM
    assert np.abs(a["p"].T - z["p"]).max() <= P_TOL
    assert np.array_equal(a["flags"], z["flags"])
    assert np.array_equal(a["mirror_shell"].astype(np.int8), z["mirror_shell"])
    assert np.array_equal(a["order"], z["order"])
    assert np.array_equal(a["ccd_num"], z["ccd_num"])
    for k in ("y_pixel", "z_pixel"):
        assert np.array_equal(a[k], z[k]), k
    assert np.array_equal(a["dither_state"][:, :3].T, z["dither_state"])
    for k in EXTRA_FIELDS:
        if k in z.files:
            got = a[k].T if k == "support_orders" else a[k]
            assert np.array_equal(got.astype(z[k].dtype), z[k]), k
    # history bits as the reference's stages set them
    want = HIST["energy"] | HIST["time"] | HIST["x"] | HIST["p"] | HIST["tag"] | HIST["shell"]
    if cfg.grating:
        want |= HIST["order"]
        if cfg.grating == cfgmod.GRATING["LETG"]:
            want |= (HIST["o1"] if cfg.leg_fine_orders else 0) | \
                    (HIST["o2"] | HIST["o3"] | HIST["o4"] if cfg.leg_coarse_orders else 0)
    if cfg.detector in (1, 2):
        want |= HIST["pixel"] | HIST["num"] | HIST["pha"] | HIST["pi"]
    elif cfg.detector in (3, 4):
        want |= HIST["region"] | HIST["pha"] | HIST["pixel"] | HIST["num"]
        if cfg.detector == 4:
            want |= HIST["uv"]
    assert hist == want, (hex(hist), hex(want))
    assert same == 1                      # the second mirror and detector calls did nothing
    good = np.nonzero((z["flags"] & 0xFF) == 0)[0]
    assert np.array_equal(idx, good)      # the final prune
    assert good.size > 0
