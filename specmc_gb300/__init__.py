"""specmc_gb300 -- the SpecMC time step on one GB300 GPU.

Drop-in surface: :class:`ConvectionConfig` and :mod:`specmc_gb300.api`
(``build_model`` / ``march`` / ``march_adaptive`` / ``production_dt`` /
``describe``), the same names and behaviour as ``specmc``.  The compute
path is ``libspecmc_gb300.so`` (hand-written sm_103a CUDA behind a C ABI,
include/specmc_gb300.h); there is no CPU fallback.
"""
from .config import ConvectionConfig  # noqa: F401
from . import api  # noqa: F401

__all__ = ["ConvectionConfig", "api"]
