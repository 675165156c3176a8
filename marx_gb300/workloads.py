"""The named photon workloads: configuration plus seeded synthetic inputs.

plain_onaxis    1e6 photons at 1.49 keV, exactly on axis, no scatter, no
                blur, no grating, no dither, ACIS-I chip/pixel.
plain_scatter   1e7 photons, log-uniform 0.3-8 keV, off-axis angle uniform
                in 0-10 arcmin at uniform azimuth, Lissajous dither 8 arcsec
                with periods 1000 s / 707 s, times uniform over 10 ks, mirror
                blur and WFold scattering, ACIS-I.
plain_hetg      2e7 photons, power law (photon index 1.7) on 0.4-8 keV
                absorbed by NH = 1e21 cm^-2, HETG orders -3..+3, ACIS-S.
plain_letg      4e6 photons of the same spectrum through the LETG and its
                support gratings, ACIS-S.
plain_hrci      4e6 photons of plain_scatter's source on the HRC-I.
letg_hrcs       4e6 photons of plain_hetg's spectrum through the LETG onto
                the HRC-S behind its Drake flat.
batched         256 sources (see marx_gb300.batched).
differentiable  4e6 weighted rays (see marx_gb300.diff).

Every input comes from numpy's PCG64 with a fixed seed per workload; no
dataset is read.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .config import MxConfig, default_config, DETECTOR, GRATING, DITHER
from .photons import PhotonList

ARCMIN = math.pi / (180.0 * 60.0)

# Smooth photo-absorption cross-section per hydrogen atom,
# sigma(E) = SIGMA_1KEV * E^(-8/3) (E in keV), normalised at 1 keV to the
# Morrison & McCammon (1983) interstellar value.
SIGMA_1KEV = 2.4e-22   # cm^2


@dataclass
class Workload:
    name: str
    n: int
    cfg: MxConfig
    seed: int
    stages: int = 15

    def photons(self, n: int | None = None, seed: int | None = None) -> PhotonList:
        """Seeded synthetic inputs (n defaults to the workload size)."""
        return GENERATORS[self.name](self, self.n if n is None else n, self.seed if seed is None else seed)


def _rng(seed):
    return np.random.default_rng(seed)


def _onaxis(w, n, seed):
    p = np.zeros((3, n)); p[0] = -1.0
    ph = PhotonList.from_inputs(np.full(n, 1.49), p)
    return ph


def offaxis_directions(theta, phi):
    """Unit vectors toward the mirror from a source theta off axis at
    azimuth phi (MARX frame: the optical axis is -X)."""
    st = np.sin(theta)
    return np.stack([-np.cos(theta), st * np.cos(phi), st * np.sin(phi)])


def _scatter(w, n, seed):
    r = _rng(seed)
    E = np.exp(r.uniform(np.log(0.3), np.log(8.0), n))
    theta = r.uniform(0.0, 10.0 * ARCMIN, n)
    phi = r.uniform(0.0, 2 * np.pi, n)
    t = r.uniform(0.0, 1e4, n)
    ph = PhotonList.from_inputs(E, offaxis_directions(theta, phi), t)
    return ph


def absorbed_powerlaw(r, n, gamma=1.7, emin=0.4, emax=8.0, nh=1e21):
    """Energies from E^-gamma * exp(-nh sigma(E)) on [emin, emax] by inverse
    transform of the power law and rejection on the absorption factor."""
    out = np.empty(0)
    a = 1.0 - gamma
    while out.size < n:
        m = int((n - out.size) * 1.6) + 1024
        u = r.random(m)
        e = (emin ** a + u * (emax ** a - emin ** a)) ** (1.0 / a)
        keep = r.random(m) < np.exp(-nh * SIGMA_1KEV * e ** (-8.0 / 3.0))
        out = np.concatenate([out, e[keep]])
    return out[:n]


def _hetg(w, n, seed):
    r = _rng(seed)
    E = absorbed_powerlaw(r, n)
    p = np.zeros((3, n)); p[0] = -1.0
    t = r.uniform(0.0, 1e4, n)
    ph = PhotonList.from_inputs(E, p, t)
    return ph


GENERATORS = {"plain_onaxis": _onaxis, "plain_scatter": _scatter, "plain_hetg": _hetg, "plain_letg": _hetg,
              "plain_hrci": _scatter, "letg_hrcs": _hetg}


def plain_onaxis(parity: bool = False) -> Workload:
    c = default_config()
    # reflectivity lookup on, everything else ideal: HRMA_Ideal=no with
    # blur, WFold and struts off (HRMA_Ideal=yes would skip reflectivity,
    # hrma.c:516)
    c.use_blur = c.use_wfold = c.use_struts = 0
    c.hrma_vig = 1.0
    c.grating = GRATING["NONE"]
    c.dither = DITHER["NONE"]
    c.detector = DETECTOR["ACIS-I"]
    c.aperture_area_uniform = 0 if parity else 1
    return Workload("plain_onaxis", 1_000_000, c, seed=101, stages=15)


def plain_scatter(parity: bool = False) -> Workload:
    c = default_config()
    c.grating = GRATING["NONE"]
    c.dither = DITHER["INTERNAL"]
    c.dither_amp[:] = [8.0, 8.0, 0.0]
    c.dither_period[:] = [1000.0, 707.0, 1e5]
    c.dither_phase[:] = [0.0, 0.0, 0.0]
    c.roll_nom = 0.0
    c.detector = DETECTOR["ACIS-I"]
    return Workload("plain_scatter", 10_000_000, c, seed=202, stages=15)


def plain_hetg(parity: bool = False) -> Workload:
    c = default_config()
    c.grating = GRATING["HETG"]
    c.max_order = 0 if parity else 3
    c.dither = DITHER["INTERNAL"]
    c.detector = DETECTOR["ACIS-S"]
    return Workload("plain_hetg", 20_000_000, c, seed=303, stages=15)


def plain_letg(parity: bool = False) -> Workload:
    """LETG with its fine and coarse support gratings, ACIS-S."""
    c = default_config()
    c.grating = GRATING["LETG"]
    c.dither = DITHER["INTERNAL"]
    c.detector = DETECTOR["ACIS-S"]
    return Workload("plain_letg", 4_000_000, c, seed=404, stages=15)


def plain_hrci(parity: bool = False) -> Workload:
    """The plain_scatter source and mirror on the HRC-I (MCP and UV/ion
    shield efficiencies, position blur, pulse height)."""
    w = plain_scatter(parity)
    w.cfg.detector = DETECTOR["HRC-I"]
    return Workload("plain_hrci", 4_000_000, w.cfg, seed=505, stages=15)


def letg_hrcs(parity: bool = False) -> Workload:
    """LETG on the HRC-S: Drake flat, MCP and shield-region efficiencies,
    u/v pixels."""
    w = plain_letg(parity)
    w.cfg.detector = DETECTOR["HRC-S"]
    return Workload("letg_hrcs", 4_000_000, w.cfg, seed=606, stages=15)


PLAIN = {"plain_onaxis": plain_onaxis, "plain_scatter": plain_scatter, "plain_hetg": plain_hetg}
# Workloads of the stages the C++ restatement does not cover (LETG, HRC):
# their parity is pinned to the reference's own outputs only.
EXTRA = {"plain_letg": plain_letg, "plain_hrci": plain_hrci, "letg_hrcs": letg_hrcs}
ALL = {**PLAIN, **EXTRA}
