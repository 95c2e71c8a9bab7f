"""The viscosity window on the host (``specmc/physics/eta_bounds.py:185-480``).

A window [eta_min, eta_max] is applied either as a hard clamp with a relative
dead-band of 1e-12 (entries inside (1 - 1e-12) eta_min ... (1 + 1e-12) eta_max
are left untouched, and the input object itself is returned when nothing is
outside) or, with a half-width w > 0 in ln eta, as the C^2 clamp
    Y = y_lo + (y - y_lo) H((y - y_lo)/w),  y_out = y_hi - (y_hi - Y) H((y_hi - Y)/w),
y = ln eta, H the quintic smoothstep 6t^5 - 15t^4 + 10t^3 on [0, 1].  The
reachable windows are the widest a law can produce over the clipped
temperature range T in [0, 2], so applying them never moves a point.  The GPU
applies the same window in its eta kernels; these are for drivers and checks.
"""
from __future__ import annotations

import math

import numpy as np

from . import _numerics as NUM
from .arrhenius import arrhenius_exponent_V, eta_arrhenius_T
from .config import validate_bounds, validate_smooth

__all__ = ["DEFAULT_MIN", "DEFAULT_MAX", "CLIP_RTOL", "SMOOTH_DEFAULT", "bounds_default",
           "reachable_window", "reachable_window_arrhenius", "reachable_window_pv",
           "effective_bounds", "validate_bounds", "clip_eta", "n_clipped", "validate_smooth",
           "smoothstep5", "n_in_transition", "smooth_clip_eta"]

DEFAULT_MIN = 1e-3
DEFAULT_MAX = 1e3
CLIP_RTOL = 1e-12
SMOOTH_DEFAULT = 0.0


def bounds_default():
    return float(DEFAULT_MIN), float(DEFAULT_MAX)


def _t_hi(t_clip):
    hi = float((NUM.ETA_T_CLIP if t_clip is None else t_clip)[1])
    if not (math.isfinite(hi) and hi >= 0.0):
        raise ValueError("temperature clip %r: its upper end must be finite and >= 0" % (t_clip,))
    return hi


def _need_positive(name, value):
    v = float(value)
    if not (math.isfinite(v) and v > 0.0):
        raise ValueError("%s: need a finite value > 0, have %r" % (name, value))
    return v


def reachable_window(deta_T, t_clip=None):
    """(deta_T^-t_hi, deta_T^t_hi): the exponential law's range over T in
    [0, t_hi], mirrored in ln eta about eta = 1."""
    d = _need_positive("deta_T", deta_T)
    hi = _t_hi(t_clip)
    return d ** (-hi), d ** hi


def reachable_window_arrhenius(deta_T, Ts, t_clip=None):
    """(eta(t_hi), 1/eta(t_hi)) of the T-only Arrhenius law."""
    d, s = _need_positive("deta_T", deta_T), _need_positive("arrhenius_Ts", Ts)
    lo = float(eta_arrhenius_T(_t_hi(t_clip), d, s))
    return lo, 1.0 / lo


def reachable_window_pv(E, V, Ts, t_clip=None):
    """(min, max) of the pV(L) law over T in [0, t_hi], p0_norm in [0, 1]:
    the hot, shallow corner and the cold, deep one."""
    lo = float(arrhenius_exponent_V(_t_hi(t_clip), 0.0, E, V, Ts, p0_norm=0.0))
    hi = float(arrhenius_exponent_V(0.0, 0.0, E, V, Ts, p0_norm=1.0))
    if not (math.isfinite(lo) and math.isfinite(hi)):
        raise ValueError("the pV window is not finite (ln eta from %r to %r)" % (lo, hi))
    return float(np.exp(lo)), float(np.exp(hi))


def effective_bounds(eta_min, eta_max):
    """The window with its dead-band: (eta_min (1 - 1e-12), eta_max (1 + 1e-12))."""
    return float(eta_min) * (1.0 - CLIP_RTOL), float(eta_max) * (1.0 + CLIP_RTOL)


def n_clipped(eta, eta_min, eta_max):
    """How many entries lie outside the window with its dead-band."""
    lo, hi = effective_bounds(eta_min, eta_max)
    e = np.asarray(eta)
    return int(((e < lo) | (e > hi)).sum())


def clip_eta(eta, eta_min, eta_max):
    """-> (eta clamped into [eta_min, eta_max], entries moved); the input
    array itself when nothing lies outside the dead-band window."""
    e = np.asarray(eta, dtype=float)
    moved = n_clipped(e, eta_min, eta_max)
    return (e, 0) if moved == 0 else (np.clip(e, eta_min, eta_max), moved)


def smoothstep5(t):
    """6t^5 - 15t^4 + 10t^3 on t clamped to [0, 1]."""
    t = np.clip(np.asarray(t, dtype=float), 0.0, 1.0)
    return t * t * t * (t * (6.0 * t - 15.0) + 10.0)


def _in_bands(y, y_lo, y_hi, w):
    return ((y > y_lo) & (y < y_lo + w)) | ((y > y_hi - w) & (y < y_hi))


def n_in_transition(eta, eta_min, eta_max, width):
    """How many entries lie strictly inside one of the two transition bands."""
    w = float(width)
    if w <= 0.0:
        return 0
    y = np.log(np.asarray(eta, dtype=float))
    return int(_in_bands(y, math.log(float(eta_min)), math.log(float(eta_max)), w).sum())


def smooth_clip_eta(eta, eta_min, eta_max, width):
    """-> (the C^2 clamp of eta, entries inside a transition band); the hard
    clamp of ``clip_eta`` when width <= 0."""
    w = float(width)
    if w <= 0.0:
        return clip_eta(eta, eta_min, eta_max)
    y_lo, y_hi = math.log(float(eta_min)), math.log(float(eta_max))
    y = np.log(np.asarray(eta, dtype=float))
    n = int(_in_bands(y, y_lo, y_hi, w).sum())
    Y = y_lo + (y - y_lo) * smoothstep5((y - y_lo) / w)
    return np.exp(y_hi - (y_hi - Y) * smoothstep5((y_hi - Y) / w)), n
