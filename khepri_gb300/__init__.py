"""khepri_gb300 — the Crystal RCWA solve path of Kaeryv/Khepri on GB300 (sm_103a) kernels.

Public API: ``Crystal`` / ``Multilayer`` / ``Layer`` (drop-in for khepri.crystal), ``batch.solve_rt``
(many problems per launch), ``workloads`` (seeded synthetic inputs), ``build.build`` (nvcc).
The compute path is libkhp (khepri_gb300/_lib/libkhp.so, C ABI in include/khepri_gb300.h).
"""
from .crystal import Crystal, Layer, Multilayer  # noqa: F401
from ._capi import KhpError  # noqa: F401

__all__ = ["Crystal", "Layer", "Multilayer", "KhpError"]
