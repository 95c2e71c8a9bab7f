"""The Arrhenius viscosity laws on the host (``specmc/physics/arrhenius.py:208-432``).

T-only law, calibrated so that eta(0) = 1 and eta(1) = 1/deta_T:
E = ln(deta_T) Ts (1 + Ts), C = -E/Ts, and ln eta evaluated in the
cancellation-free form -ln(deta_T) (1 + Ts) T / (T + Ts).  Pressure-dependent
law pV(L): ln eta = -E T / (Ts (T + Ts)) + V p0_norm / (T + Ts) with
p0_norm = 1 - z.  Plus the slope and contrast diagnostics and the inverse
calibrations.  The GPU evaluates the same two forms in its eta kernel."""
from __future__ import annotations

import math

import numpy as np

from .config import arrhenius_derived_E as arrhenius_E
from .reference_state import p0_norm as _p0_norm

__all__ = ["arrhenius_E", "arrhenius_C", "arrhenius_exponent", "eta_arrhenius_T",
           "arrhenius_exponent_V", "eta_arrhenius_V", "hot_end_contrast_V", "cold_end_slope",
           "slope_amplification", "infer_deta_T", "infer_Ts"]


def _positive(name, value):
    v = float(value)
    if not (math.isfinite(v) and v > 0.0):
        raise ValueError("%s: need a finite value > 0, have %r" % (name, value))
    return v


def arrhenius_C(deta_T, Ts):
    """C = -E/Ts = -ln(deta_T) (1 + Ts)."""
    return -arrhenius_E(deta_T, Ts) / float(Ts)


def arrhenius_exponent(T, deta_T, Ts):
    """ln eta(T) = -ln(deta_T) (1 + Ts) T / (T + Ts)."""
    T = np.asarray(T, dtype=float)
    s = float(Ts)
    return -float(np.log(float(deta_T))) * (1.0 + s) * T / (T + s)


def eta_arrhenius_T(T, deta_T, Ts):
    """exp(arrhenius_exponent(T, deta_T, Ts))."""
    return np.exp(arrhenius_exponent(T, deta_T, Ts))


def arrhenius_exponent_V(T, z, E, V, Ts, p0_norm=None):
    """ln eta of the pV(L) law, -E T / (Ts (T + Ts)) + V p0 / (T + Ts), with
    p0 = ``p0_norm`` or 1 - z."""
    s = _positive("Ts", Ts)
    E, V = float(E), float(V)
    for name, value in (("E", E), ("V", V)):
        if not math.isfinite(value):
            raise ValueError("%s must be finite, have %r" % (name, value))
    T = np.asarray(T, dtype=float)
    p0 = _p0_norm(z) if p0_norm is None else np.asarray(p0_norm, dtype=float)
    return -E * T / (s * (T + s)) + V * p0 / (T + s)


def eta_arrhenius_V(T, z, E, V, Ts, p0_norm=None):
    """exp(arrhenius_exponent_V(...))."""
    return np.exp(arrhenius_exponent_V(T, z, E, V, Ts, p0_norm=p0_norm))


def hot_end_contrast_V(T, z, E, V, Ts, p0_norm=None):
    """max eta / min eta of the pV(L) field over the given points."""
    g = np.asarray(arrhenius_exponent_V(T, z, E, V, Ts, p0_norm=p0_norm))
    return float(np.exp(float(g.max()) - float(g.min())))


def cold_end_slope(deta_T, Ts):
    """|d ln eta / dT| at T = 0: E / Ts^2."""
    return arrhenius_E(deta_T, Ts) / float(Ts) ** 2


def slope_amplification(Ts):
    """The cold-end slope in units of ln(deta_T): (1 + Ts) / Ts."""
    s = _positive("arrhenius_Ts", Ts)
    return (1.0 + s) / s


def infer_deta_T(E, Ts):
    """The contrast a calibrated activation implies: exp(E / (Ts (1 + Ts)))."""
    E, s = _positive("E", E), _positive("arrhenius_Ts", Ts)
    return float(np.exp(E / (s * (1.0 + s))))


def infer_Ts(E, deta_T):
    """The positive Ts with E = ln(deta_T) Ts (1 + Ts)."""
    E = _positive("E", E)
    D = float(deta_T)
    if not (math.isfinite(D) and D > 1.0):
        raise ValueError("deta_T: need a finite value > 1, have %r" % (deta_T,))
    return float(0.5 * (math.sqrt(1.0 + 4.0 * E / math.log(D)) - 1.0))
