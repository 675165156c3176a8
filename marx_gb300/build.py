"""Build libmarx_gb300.so in-tree for sm_103a (GB300).

    python -m marx_gb300.build [--verbose]

Each translation unit is compiled by nvcc in parallel, then linked into
marx_gb300/_build/libmarx_gb300.so.  Host files are compiled by nvcc too so
that one toolchain builds the whole library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmarx_gb300.so")
# MARX's own stage API over its array-of-structures photon list
# (include/marx_gb300_compat.h), on top of LIB
COMPAT_LIB = os.path.join(OUT, "libmarx_gb300_compat.so")
COMPAT_SOURCES = ["mx_compat.cpp"]
SOURCES = ["mx_capi.cu", "mx_kernels.cu", "mx_batch.cu", "mx_static.cu", "mx_diff.cu", "mx_model.cpp",
           "mx_output.cpp", "mx_source.cpp", "mx_events.cu", "mx_user_source.cpp", "mx_par.cpp", "mx_run.cu", "mx_saosac.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags(src: str, verbose: bool):
    # host code: no fused multiply-add contraction (gcc contracts by default on
    # aarch64), so the init-time tables round as the reference's do
    f = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-lineinfo",
         "--expt-relaxed-constexpr"]
    if src.endswith(".cu"):
        f += ARCH
        if os.path.basename(src) == "mx_events.cu":
            # no multiply-add contraction: DETX/DETY round like the reference's
            f += ["--fmad=false"]
        if verbose:
            f += ["-Xptxas", "-v"]
    else:
        f += ["-x", "c++"]
    return f


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    compat = [os.path.join(CSRC, s) for s in COMPAT_SOURCES]
    inc = os.path.join(os.path.dirname(HERE), "include")
    deps = srcs + compat + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps += [os.path.join(inc, h) for h in os.listdir(inc)]
    if (not force and all(os.path.exists(f) for f in (LIB, COMPAT_LIB))
            and all(min(os.path.getmtime(LIB), os.path.getmtime(COMPAT_LIB)) >= os.path.getmtime(d) for d in deps)):
        return LIB
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        cmd = [cc, *_flags(src, verbose), "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(len(srcs) + len(compat)) as ex:
        objs = list(ex.map(compile_one, srcs + compat))
    core, shim = objs[:len(srcs)], objs[len(srcs):]
    for out, cmd in ((LIB, [*ARCH, "-shared", *core, "-lcudart", "-ldl"]),
                     (COMPAT_LIB, ["-shared", *shim, "-L" + OUT, "-lmarx_gb300", "-lcudart", "-ldl",
                                   "-Xlinker", "-rpath,$ORIGIN"])):
        tmp = out + ".tmp"
        r = subprocess.run([cc, "-o", tmp, *cmd], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of {os.path.basename(out)} failed:\n{r.stderr}")
        os.replace(tmp, out)
    return LIB


if __name__ == "__main__":
    print(build(verbose="--verbose" in sys.argv, force=True))
