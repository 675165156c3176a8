"""The compatibility shim without a GPU: the layout of the reference's
photon types in include/marx_gb300_compat.h against the reference's own
marx.h, the library's exports, the host-side pieces (allocation,
marx_prune_photons, errors before initialisation), and the reference's
unmodified marx program linked against the shim."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "marx_gb300_compat.h")

ATTR_FIELDS = ["energy", "x", "p", "arrival_time", "flags", "y_pixel", "z_pixel", "u_pixel", "v_pixel",
               "dither_state", "pi", "pulse_height", "mirror_shell", "ccd_num", "detector_region", "order",
               "support_orders", "tag"]
TYPE_FIELDS = ["source_distance", "attributes", "n_photons", "max_n_photons", "total_time", "start_time",
               "sorted_index", "sorted_energies", "num_sorted", "history", "tag_start"]
DITHER_FIELDS = ["ra", "dec", "roll", "dy", "dz", "dtheta"]

# Marx_Photon_Attr_Type as numpy sees it (C alignment rules)
ATTR_DTYPE = np.dtype([("energy", "f8"), ("x", "f8", 3), ("p", "f8", 3), ("arrival_time", "f8"), ("flags", "u4"),
                       ("y_pixel", "f4"), ("z_pixel", "f4"), ("u_pixel", "f4"), ("v_pixel", "f4"),
                       ("dither_state", "f4", 6), ("pi", "f4"), ("pulse_height", "i2"), ("mirror_shell", "u4"),
                       ("ccd_num", "i1"), ("detector_region", "i1"), ("order", "i1"), ("support_orders", "i1", 4),
                       ("tag", "u4")], align=True)


def _layout(tmp_path, header, incs):
    src = tmp_path / "layout.c"
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{header}"',
             "#define F(s, m) printf(#s \".\" #m \" %zu %zu\\n\", offsetof(s, m), sizeof(((s *) 0)->m))",
             "int main(void) {",
             'printf("sizeof %zu %zu %zu\\n", sizeof(Marx_Photon_Attr_Type), sizeof(Marx_Photon_Type), '
             'sizeof(Marx_Dither_Type));']
    lines += [f"F(Marx_Photon_Attr_Type, {f});" for f in ATTR_FIELDS]
    lines += [f"F(Marx_Photon_Type, {f});" for f in TYPE_FIELDS]
    lines += [f"F(Marx_Dither_Type, {f});" for f in DITHER_FIELDS]
    lines += ["return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", *[f"-I{i}" for i in incs], str(src), "-o", str(exe)], check=True)
    return subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout


def test_photon_types_have_the_reference_layout(tmp_path):
    """offsetof and sizeof of every member of Marx_Photon_Attr_Type,
    Marx_Photon_Type and Marx_Dither_Type: the shim's declarations against
    the reference's marx.h (marx.h:42-151) compiled by the same compiler."""
    from oracle.bindings import REF_ROOT, reference_available
    ours = _layout(tmp_path, "marx_gb300_compat.h", [os.path.join(ROOT, "include")])
    sizes = ours.splitlines()[0].split()
    assert sizes[1:] == ["136", "80", "24"]
    # numpy's aligned record, as the GPU test reads the attributes back
    offs = {l.split()[0].split(".")[1]: int(l.split()[1]) for l in ours.splitlines()[1:]
            if l.startswith("Marx_Photon_Attr_Type.")}
    assert ATTR_DTYPE.itemsize == 136
    assert all(ATTR_DTYPE.fields[k][1] == offs[k] for k in ATTR_FIELDS)
    if not reference_available():
        pytest.skip("the reference checkout is not on this machine")
    ref = _layout(tmp_path, "marx.h", [os.path.join(REF_ROOT, "marx", "libsrc"), os.path.join(REF_ROOT, "jdmath", "src"),
                                        os.path.join(REF_ROOT, "pfile", "src"), os.path.join(ROOT, "oracle", "ref_config")])
    assert ours == ref


def declared_functions():
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    return sorted(set(re.findall(r"\b(marx_[a-z0-9_]+)\s*\(", txt)))


def _compat():
    from marx_gb300.build import build, COMPAT_LIB
    build()
    return C.CDLL(COMPAT_LIB)


def test_compat_library_exports_every_declared_function():
    L = _compat()
    names = declared_functions()
    assert {"marx_mirror_reflect", "marx_grating_diffract", "marx_detect", "marx_prune_photons"} <= set(names)
    for n in names:
        assert hasattr(L, n), n


class PhotonType(C.Structure):
    _fields_ = [("source_distance", C.c_double), ("attributes", C.c_void_p), ("n_photons", C.c_uint),
                ("max_n_photons", C.c_uint), ("total_time", C.c_double), ("start_time", C.c_double),
                ("sorted_index", C.POINTER(C.c_uint)), ("sorted_energies", C.POINTER(C.c_double)),
                ("num_sorted", C.c_uint), ("history", C.c_ulong), ("tag_start", C.c_uint)]


def _batch(L, n):
    L.marx_alloc_photon_type.restype = C.POINTER(PhotonType)
    L.marx_alloc_photon_type.argtypes = [C.c_uint]
    pt = L.marx_alloc_photon_type(n)
    assert pt
    buf = (C.c_char * (136 * n)).from_address(pt.contents.attributes)
    attrs = np.frombuffer(buf, dtype=ATTR_DTYPE)
    return pt, attrs


def test_prune_keeps_good_photons_in_order():
    """marx_prune_photons (photon.c:40-62): sorted_index keeps the photons
    without a BAD_PHOTON_MASK bit in their order, sorted_energies follows."""
    L = _compat()
    n = 1000
    pt, attrs = _batch(L, n)
    rng = np.random.default_rng(3)
    attrs["energy"] = rng.uniform(0.3, 8, n)
    attrs["flags"] = rng.choice([0, 0, 0x02, 0x08, 0x100, 0x200, 0x80], n)
    order = rng.permutation(n).astype(np.uint32)
    p = pt.contents
    for i in range(n):
        p.sorted_index[i] = int(order[i])
    p.num_sorted = n
    p.n_photons = n
    L.marx_prune_photons(pt)
    keep = [int(k) for k in order if (attrs["flags"][k] & 0xFF) == 0]
    assert p.num_sorted == len(keep)
    assert [p.sorted_index[i] for i in range(p.num_sorted)] == keep
    assert np.array_equal([p.sorted_energies[i] for i in range(p.num_sorted)], attrs["energy"][keep])
    L.marx_prune_photons(pt)          # idempotent
    assert p.num_sorted == len(keep)
    assert L.marx_dealloc_photon_type(pt) == 0


def test_stages_refuse_before_init_and_without_a_parameter_library():
    L = _compat()
    L.marx_gb300_compat_last_error.restype = C.c_char_p
    pt, _ = _batch(L, 4)
    for f, msg in (("marx_mirror_reflect", b"Mirror not initialized"), ("marx_grating_diffract", b"Grating"),
                   ("marx_detect", b"Detector")):
        assert getattr(L, f)(pt, 0) == -1
        assert msg in L.marx_gb300_compat_last_error()
    # this process links no pf_get_*: every *_init says so
    assert L.marx_mirror_init(None) == -1
    assert b"parameter-file library" in L.marx_gb300_compat_last_error()
    assert L.marx_gb300_compat_set_variates(C.c_void_p(8), None, 4) == -1
    L.marx_dealloc_photon_type(pt)


def test_stock_marx_binds_its_stage_calls_to_the_shim(tmp_path):
    """The reference's own marx program (marx/src/marx.c, unmodified),
    compiled and linked with libmarx_gb300_compat ahead of the reference's
    modules (oracle/Makefile target marx): its stage calls and the
    mirror-module globals the source reads bind to the shim, and a run gets
    through the parameter file, the shim's *_init functions and the
    reference's source up to the first stage, which asks the engine for a
    GPU (on a machine without one it stops there with the shim's error)."""
    from oracle.bindings import REF_ROOT, reference_available
    if not reference_available():
        pytest.skip("the reference checkout is not on this machine")
    _compat()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "marx", f"REF={REF_ROOT}"], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "marx_gb300")
    par = tmp_path / "marx.par"
    par.write_text(open(os.path.join(REF_ROOT, "marx", "par", "marx.par")).read())
    env = dict(os.environ, MARX_DATA_DIR=os.path.join(REF_ROOT, "marx", "data"), LD_DEBUG="bindings",
               LD_BIND_NOW="1", LD_DEBUG_OUTPUT=str(tmp_path / "ld"))
    r = subprocess.run([exe, "NumRays=1000", "dNumRays=1000", f"OutputDir={tmp_path / 'out'}", "DetectorType=ACIS-I",
                        "GratingType=NONE", f"DataDirectory={os.path.join(REF_ROOT, 'marx', 'data')}"],
                       cwd=tmp_path, env=env, capture_output=True, text=True, timeout=120)
    log = "".join(open(os.path.join(tmp_path, f)).read() for f in os.listdir(tmp_path) if f.startswith("ld"))
    for sym in ("marx_mirror_reflect", "marx_grating_diffract", "marx_detect", "marx_prune_photons",
                "marx_mirror_init", "marx_detector_init", "Marx_Mirror_Geometric_Area"):
        binds = [ln for ln in log.splitlines() if f"symbol `{sym}'" in ln]
        assert binds and all("libmarx_gb300_compat.so" in ln.split(" to ")[1] for ln in binds), sym
    out = r.stdout + r.stderr
    assert "1000 photons collected" in out
    import torch
    if not torch.cuda.is_available():
        assert "(gb300 compat) error: creating the engine" in out
