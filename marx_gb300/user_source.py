"""USER sources (marx/libsrc/s-user.c): a MARX user-source plug-in driven
through the engine's C ABI (mx_user_source_open / _create / _close).  The
plug-in's rays fill a host PhotonList that is then traced like any other."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .photons import MxPhotons, PhotonList


def _lib():
    from ._native import load_library
    L = load_library()
    if not getattr(L, "_mx_user_bound", False):
        L.mx_user_source_open.restype = C.c_void_p
        L.mx_user_source_open.argtypes = [C.c_char_p, C.c_char_p, C.c_double, C.POINTER(C.c_double * 3)]
        L.mx_user_source_create.argtypes = [C.c_void_p, C.POINTER(MxPhotons), C.c_uint32, C.POINTER(C.c_uint32),
                                            C.POINTER(C.c_int)]
        L.mx_user_source_close.argtypes = [C.c_void_p]
        L.mx_user_source_error.restype = C.c_char_p
        L._mx_user_bound = True
    return L


class UserSource:
    """UserSourceFile / UserSourceArgs of marx.par, opened with the mirror's
    geometric area (cm^2) and the source direction p."""

    def __init__(self, path: str, args: str = "", geometric_area: float = 1.0, p=(-1.0, 0.0, 0.0)):
        self.L = _lib()
        self.h = self.L.mx_user_source_open(path.encode(), args.encode(), geometric_area,
                                            C.byref((C.c_double * 3)(*p)))
        if not self.h:
            raise RuntimeError("user source: " + self.L.mx_user_source_error().decode())

    def create(self, energies) -> tuple[PhotonList, bool]:
        """Photons for the spectrum's energy draws `energies`: the list (as
        many photons as the plug-in made) and whether it set arrival times."""
        e = np.ascontiguousarray(energies, dtype=np.float64)
        ph = PhotonList(len(e))
        ph.energy[:] = e
        s = ph.struct()
        got, ts = C.c_uint32(0), C.c_int(0)
        if self.L.mx_user_source_create(self.h, C.byref(s), len(e), C.byref(got), C.byref(ts)) != 0:
            raise RuntimeError("user source: " + self.L.mx_user_source_error().decode())
        m = got.value
        q = PhotonList(m)
        for k in ("energy", "p", "arrival_time", "flags"):
            setattr(q, k, np.ascontiguousarray(getattr(ph, k)[..., :m]))
        return q, bool(ts.value)

    def close(self):
        if self.h:
            self.L.mx_user_source_close(self.h)
            self.h = None
