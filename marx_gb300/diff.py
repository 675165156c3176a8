"""Differentiable form: weighted-ray focal-plane images and their adjoint
(mx_diff_* in include/marx_gb300.h).

    eng = Engine(diff_mirror_config())
    w = diff_workload()                       # 4e6 rays, 1.49 keV, 2' off-axis
    img = DiffImage.centred(eng, w.cfg)       # image centred on the PSF
    I = img.forward(theta)                    # device (256, 256) float64
    loss, dl = img.mse(I, target)
    g = img.adjoint(theta, dl)                # numpy (18,)

theta[4 s + 0..3] are shell s's az_mis and el_mis (arcsec) and x0 and y0
(micrometres), added to both its P and H rows; theta[16..17] the source
offset in y and z (arcsec).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from .config import MxConfig, default_config, DITHER, GRATING, DETECTOR

NPARAM = 18
RECORD, REPLAY, FRESH = 0, 1, 2
PARAM_NAMES = [f"shell{s}_{k}" for s in (1, 3, 4, 6) for k in ("az", "el", "x0", "y0")] + ["src_y", "src_z"]
ARCSEC = math.pi / (180.0 * 3600.0)


class MxDiffConfig(C.Structure):
    _fields_ = [("n_rays", C.c_uint64), ("seed", C.c_uint64), ("energy", C.c_double),
                ("src_y", C.c_double), ("src_z", C.c_double), ("center_y", C.c_double),
                ("center_z", C.c_double), ("pitch", C.c_double), ("sigma", C.c_double),
                ("nx", C.c_uint32), ("ny", C.c_uint32)]

    def copy(self) -> "MxDiffConfig":
        c = MxDiffConfig()
        C.pointer(c)[0] = self
        return c


def _bind(L):
    if getattr(L, "_diff_bound", False):
        return L
    L.mx_diff_create.restype = C.c_void_p
    L.mx_diff_create.argtypes = [C.c_void_p, C.POINTER(MxDiffConfig)]
    L.mx_diff_destroy.argtypes = [C.c_void_p]
    dp = C.POINTER(C.c_double)
    L.mx_diff_forward.argtypes = [C.c_void_p, dp, C.c_int, C.c_void_p, dp, C.c_void_p]
    L.mx_diff_rays.argtypes = [C.c_void_p, dp, C.c_int, C.c_void_p, C.c_void_p]
    L.mx_diff_mse.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.mx_diff_adjoint.argtypes = [C.c_void_p, dp, C.c_void_p, dp, C.c_void_p]
    L.mx_diff_adjoint_async.argtypes = [C.c_void_p, dp, C.c_void_p, C.c_void_p, C.c_void_p]
    L._diff_bound = True
    return L


def _theta(theta) -> C.Array:
    t = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).reshape(-1))
    if t.size != NPARAM:
        raise ValueError(f"theta must have {NPARAM} entries")
    return (C.c_double * NPARAM)(*t.tolist())


def source_direction(src_y: float, src_z: float) -> np.ndarray:
    """Unit direction of travel of a source at tangent-plane angles
    (src_y, src_z) arcsec: unit(-1, -tan y, -tan z)."""
    v = np.array([-1.0, -math.tan(src_y * ARCSEC), -math.tan(src_z * ARCSEC)])
    return v / math.sqrt(float(v @ v))


class DiffImage:
    """One mx_diff handle: weighted rays of one source over the engine's
    mirror model, imaged on an nx x ny grid."""

    def __init__(self, engine, cfg: MxDiffConfig):
        self.eng = engine
        self.L = _bind(engine.lib)
        self.cfg = cfg.copy()
        self.h = self.L.mx_diff_create(engine.h, C.byref(self.cfg))
        if not self.h:
            raise RuntimeError("mx_diff_create: " + self.L.mx_last_error(engine.h).decode())

    @classmethod
    def centred(cls, engine, cfg: MxDiffConfig, theta=None):
        """A handle whose image centre is the weighted centroid of the rays
        at theta (default 0)."""
        probe = cls(engine, cfg)
        mom = probe.moments(np.zeros(NPARAM) if theta is None else theta)
        probe.close()
        c = cfg.copy()
        c.center_y = mom[1] / mom[0]
        c.center_z = mom[2] / mom[0]
        return cls(engine, c)

    def close(self):
        if getattr(self, "h", None):
            self.L.mx_diff_destroy(self.h)
            self.h = None

    __del__ = close

    def _check(self, r):
        if r != 0:
            raise RuntimeError(f"marx_gb300 error {r}: " + self.L.mx_last_error(self.eng.h).decode())

    @staticmethod
    def _stream(stream):
        import torch
        return (stream if stream is not None else torch.cuda.current_stream()).cuda_stream

    def new_image(self):
        import torch
        return torch.empty((self.cfg.ny, self.cfg.nx), dtype=torch.float64, device="cuda")

    def forward(self, theta, mode: int = RECORD, out=None, stream=None):
        """The image at theta (device float64 tensor, rows = z)."""
        img = self.new_image() if out is None else out
        self._check(self.L.mx_diff_forward(self.h, _theta(theta), mode, C.c_void_p(img.data_ptr()), None,
                                           C.c_void_p(self._stream(stream))))
        return img

    def moments(self, theta, mode: int = FRESH):
        """(sum w, sum w y, sum w z, rays reaching the focal plane)."""
        img = self.new_image()
        m = (C.c_double * 4)()
        self._check(self.L.mx_diff_forward(self.h, _theta(theta), mode, C.c_void_p(img.data_ptr()), m,
                                           C.c_void_p(self._stream(None))))
        return np.array(m[:])

    def rays(self, theta, mode: int = FRESH, stream=None):
        """Per-ray focal-plane y, z (mm) and weight w: device tensor (3, n)."""
        import torch
        yzw = torch.empty((3, self.cfg.n_rays), dtype=torch.float64, device="cuda")
        self._check(self.L.mx_diff_rays(self.h, _theta(theta), mode, C.c_void_p(yzw.data_ptr()),
                                        C.c_void_p(self._stream(stream))))
        return yzw

    def mse(self, image, target, want_grad: bool = True, loss=None, stream=None):
        """(loss, dl/dimage): a device scalar tensor and a device image (None
        without want_grad)."""
        import torch
        loss = torch.empty((), dtype=torch.float64, device="cuda") if loss is None else loss
        dl = torch.empty_like(image) if want_grad else None
        self._check(self.L.mx_diff_mse(self.h, C.c_void_p(image.data_ptr()), C.c_void_p(target.data_ptr()),
                                       C.c_void_p(dl.data_ptr()) if dl is not None else None,
                                       C.c_void_p(loss.data_ptr()), C.c_void_p(self._stream(stream))))
        return loss, dl

    def adjoint(self, theta, dl_dimage, stream=None) -> np.ndarray:
        """d(loss)/d(theta) for dl_dimage = d(loss)/d(image) (device)."""
        g = (C.c_double * NPARAM)()
        dl = dl_dimage.contiguous()
        self._check(self.L.mx_diff_adjoint(self.h, _theta(theta), C.c_void_p(dl.data_ptr()), g,
                                           C.c_void_p(self._stream(stream))))
        return np.array(g[:])

    def adjoint_async(self, theta, dl_dimage, grad_out, stream=None):
        """Device form: grad_out is a device float64 tensor of NPARAM."""
        self._check(self.L.mx_diff_adjoint_async(self.h, _theta(theta), C.c_void_p(dl_dimage.data_ptr()),
                                                 C.c_void_p(grad_out.data_ptr()), C.c_void_p(self._stream(stream))))
        return grad_out


def fd_gradient(img: DiffImage, theta, target, h=2e-3, mode: int = REPLAY, stream=None) -> np.ndarray:
    """Central finite differences of mse(image(theta), target): 2 NPARAM
    forward images, losses kept on the device, one wait at the end."""
    import torch
    theta = np.asarray(theta, dtype=np.float64)
    hv = np.broadcast_to(np.asarray(h, dtype=np.float64), (NPARAM,))
    losses = torch.empty(2 * NPARAM, dtype=torch.float64, device="cuda")
    buf = img.new_image()
    for k in range(NPARAM):
        for j, sgn in enumerate((-1.0, 1.0)):
            t = theta.copy()
            t[k] += sgn * hv[k]
            img.forward(t, mode, out=buf, stream=stream)
            img.mse(buf, target, want_grad=False, loss=losses[2 * k + j], stream=stream)
    L = losses.cpu().numpy()
    return (L[1::2] - L[0::2]) / (2.0 * hv)


def diff_mirror_config(ideal: bool = False) -> MxConfig:
    """The mirror model the weighted rays use: the default HRMA (struts,
    reflectivity and correction factors), no dither, grating or detector
    (rays end on the focal plane)."""
    c = default_config()
    c.dither = DITHER["NONE"]
    c.grating = GRATING["NONE"]
    c.detector = DETECTOR["ACIS-I"]
    c.hrma_ideal = 1 if ideal else 0
    return c


@dataclass
class DiffWorkload:
    cfg: MxDiffConfig
    theta_true: np.ndarray   # seeded perturbation that makes the target image
    target_seed: int


def diff_workload(n_rays: int = 4_000_000, seed: int = 5, perturb_seed: int = 55) -> DiffWorkload:
    """Differentiable-form workload: n_rays weighted rays at 1.49 keV from a
    source 2' off-axis; 256 x 256 image of 24 um pixels, Gaussian sigma 1
    pixel; the target is made at theta_true, per-shell tilts N(0, 2"),
    decenters N(0, 10 um) and a source offset N(0, 0.5"), with rays of
    another seed."""
    c = MxDiffConfig()
    c.n_rays = n_rays
    c.seed = seed
    c.energy = 1.49
    c.src_y = 120.0
    c.src_z = 0.0
    c.center_y = 0.0
    c.center_z = 0.0
    c.pitch = 0.024
    c.sigma = 1.0
    c.nx = 256
    c.ny = 256
    r = np.random.default_rng(perturb_seed)
    t = np.zeros(NPARAM)
    for s in range(4):
        t[4 * s + 0] = r.normal(0.0, 2.0)
        t[4 * s + 1] = r.normal(0.0, 2.0)
        t[4 * s + 2] = r.normal(0.0, 10.0)
        t[4 * s + 3] = r.normal(0.0, 10.0)
    t[16] = r.normal(0.0, 0.5)
    t[17] = r.normal(0.0, 0.5)
    return DiffWorkload(c, t, seed + 1000)


def main(argv=None):
    """Gradient steps of the differentiable workload on the current GPU:
    python -m marx_gb300.diff [--rays N] [--steps K]"""
    import argparse
    import torch
    from ._native import Engine
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--rays", type=int, default=4_000_000)
    ap.add_argument("--steps", type=int, default=2)
    a = ap.parse_args(argv)
    eng = Engine(diff_mirror_config())
    w = diff_workload(n_rays=a.rays)
    d = DiffImage.centred(eng, w.cfg)
    tc = d.cfg.copy()
    tc.seed = w.target_seed
    target = DiffImage(eng, tc).forward(w.theta_true, FRESH).clone()
    theta = np.zeros(NPARAM)
    for _ in range(a.steps):
        img = d.forward(theta, RECORD)
        loss, dl = d.mse(img, target)
        g = d.adjoint(theta, dl)
    torch.cuda.synchronize()
    print(f"loss {float(loss):.6e}")
    for name, v in zip(PARAM_NAMES, g):
        print(f"{name:>10s} {v: .6e}")


if __name__ == "__main__":
    main()
