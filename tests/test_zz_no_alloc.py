"""mx_trace_static: the trace entry point for callers that cannot allocate
device memory while tracing (its survivor queues live in a device array
built into the library).  Called through the C ABI and checked against
mx_trace on the same photons, twice in a row, since every call reuses the
same array and must start from cleared queue counters."""
import ctypes as C

import numpy as np
import pytest

from marx_gb300 import workloads as W
from marx_gb300.photons import MxPhotons, MxVariates

from helpers import assert_parity

pytestmark = pytest.mark.gpu


def _bind():
    from marx_gb300._native import load_library
    L = load_library()
    L.mx_trace_static.argtypes = [C.c_void_p, C.POINTER(MxPhotons), C.c_uint32, C.POINTER(MxVariates),
                                  C.c_uint64, C.c_void_p]
    return L


def test_static_scratch_trace_matches_mx_trace(cuda):
    import torch
    from marx_gb300._native import Engine, DevicePhotons, MODE_WAVEFRONT
    L = _bind()
    w = W.plain_hetg()
    eng = Engine(w.cfg)               # fresh: no wavefront queues allocated yet
    eng.set_mode(MODE_WAVEFRONT)
    ph = w.photons(100_000, seed=2024)
    lists = [DevicePhotons.from_host(ph) for _ in range(2)]
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    free = []
    for d in lists:
        s = d.struct()
        rc = L.mx_trace_static(eng.h, C.byref(s), 15, C.byref(MxVariates(None, None)), 17, C.c_void_p(stream))
        assert rc == 0, L.mx_last_error(eng.h).decode()
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
    # the first call may load the kernels' module; the second allocates nothing
    assert free[1] == free[0]

    ref = DevicePhotons.from_host(ph)
    eng.trace(ref, seed=17)
    torch.cuda.synchronize()
    expected = ref.to_host()
    for call, d in enumerate(lists):
        assert_parity(d.to_host(), expected, f"static scratch, call {call + 1}")
    assert ((expected.flags & 0xFF) == 0).sum() > 1000


def test_static_scratch_rejects_lists_beyond_its_size(cuda):
    from marx_gb300._native import Engine, DevicePhotons
    L = _bind()
    eng = Engine(W.plain_onaxis().cfg)
    d = DevicePhotons(16)
    s = d.struct()
    s.n = 131072 + 1
    rc = L.mx_trace_static(eng.h, C.byref(s), 15, None, 1, None)
    assert rc == -5 and b"exceed" in L.mx_last_error(eng.h)
