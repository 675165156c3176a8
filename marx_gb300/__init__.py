"""marx_gb300: GB300-native photon trace for MARX's stage pipeline.

The engine is the C ABI library ``libmarx_gb300.so`` (include/marx_gb300.h)
built from ``marx_gb300/csrc``; this package is a thin host-side mirror of
the reference's stage API over it (``marx_gb300._native``: ``Engine``,
``DevicePhotons``) plus the table pack builder, parameter handling and
workload definitions.
"""
from .config import MxConfig, default_config, from_par, to_par  # noqa: F401
from .photons import PhotonList  # noqa: F401
