"""Source models on the GPU (mx_generate_source) against the reference's
own create_photons functions (POINT, GAUSS, BETA, DISK, LINE, IMAGE; FLAT and
FILE spectra) fed the same uniforms: tests/golden/sources.npz.  Energies exact;
directions within 1e-12 (library sine and cosine of the same arguments)."""
import os

import numpy as np
import pytest

from marx_gb300 import batched as B

from helpers import GOLDEN, P_TOL, assert_parity

pytestmark = pytest.mark.gpu
CASES = {"point": "POINT", "gauss": "GAUSS", "beta": "BETA", "disk": "DISK", "line": "LINE", "gauss_file": "GAUSS",
         "image": "IMAGE"}


def fixture():
    return np.load(os.path.join(GOLDEN, "sources.npz"))


def source_of(z, name, n):
    spec = (z["spectrum_energy"], z["spectrum_flux"]) if name.endswith("_file") else None
    return B.make_source(z[f"{name}_src"], CASES[name], tuple(z[f"{name}_param"]), energy=(0.5, 7.0),
                         spectrum=spec, num_photons=n, image=z["image"] if name == "image" else None)


def generate(eng, src, n, seed, first_tag=0):
    import torch
    from marx_gb300._native import DevicePhotons
    d = DevicePhotons(n)
    B.generate_source(eng, src, first_tag, seed, d)
    torch.cuda.synchronize()
    return d.to_host()


@pytest.mark.parametrize("name", list(CASES))
def test_source_model_matches_reference(cuda, name):
    from marx_gb300._native import Engine
    z = fixture()
    n = int(z["n"])
    eng = Engine(B.batched_config())
    q = generate(eng, source_of(z, name, n), n, int(z["seed"]))
    assert np.array_equal(q.energy, z[f"{name}_energy"]), name
    assert np.abs(q.p - z[f"{name}_p"]).max() <= P_TOL, (name, np.abs(q.p - z[f"{name}_p"]).max())
    assert np.array_equal(q.tag, np.arange(n, dtype=np.uint32))


def test_mixed_model_batch_equals_sequential(cuda):
    import ctypes as C
    import torch
    from marx_gb300._native import Engine
    z = fixture()
    srcs = (B.MxSource * len(CASES))()
    keep = []
    for k, name in enumerate(CASES):
        s = source_of(z, name, 3000 + 1000 * k)
        s.detector = B.DETECTOR["ACIS-I"]
        keep.append(s)
        C.pointer(srcs[k])[0] = s
    eng = Engine(B.batched_config())
    b = B.Batch(eng, srcs)
    b.run(seed=11)
    torch.cuda.synchronize()
    one = b.to_host()
    b.run_sequential(seed=11)
    torch.cuda.synchronize()
    seq = b.to_host()
    assert np.array_equal(one.energy, seq.energy)
    assert_parity(one, seq, "mixed models batched vs sequential")


def test_bad_source_parameters_are_rejected(cuda):
    from marx_gb300._native import Engine
    z = fixture()
    eng = Engine(B.batched_config())
    s = source_of(z, "beta", 10)
    s.param[1] = 0.4                       # beta <= 1/2
    with pytest.raises(RuntimeError, match="Beta parameters"):
        generate(eng, s, 10, 1)
