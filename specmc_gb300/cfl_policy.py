"""The production step-size policy (``specmc/core/cfl_policy.py:40-73``).

dt = min(dtmax, model.cfl_dt(that, safety=clamp(safety), dtmax, dtmin)), with
the safety factor clamped into [0, CFL_SAFETY_MAX] so that a larger request
can never lift dt above the cap.  ``api.production_dt`` and the models'
``production_dt`` / device march apply the same policy on the GPU.
"""
from __future__ import annotations

from . import _numerics as NUM

__all__ = ["CFL_SAFETY_DEFAULT", "CFL_SAFETY_MAX", "clamp_safety", "cfl_dt"]

CFL_SAFETY_DEFAULT = float(NUM.CFL_SAFETY)
CFL_SAFETY_MAX = float(NUM.CFL_MAX)


def clamp_safety(safety, lo=0.0):
    """``safety`` limited to [lo, CFL_SAFETY_MAX]."""
    return min(max(float(safety), float(lo)), CFL_SAFETY_MAX)


def cfl_dt(model, that, safety=CFL_SAFETY_DEFAULT, dtmax=4.0e-5, dtmin=1e-10, clamp=True):
    """The policy's dt for ``that`` on ``model`` (``clamp=False`` passes
    ``safety`` through unchanged)."""
    fac = clamp_safety(safety) if clamp else float(safety)
    return float(min(dtmax, model.cfl_dt(that, safety=fac, dtmax=dtmax, dtmin=dtmin)))
