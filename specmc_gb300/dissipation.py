"""``specmc.physics.dissipation`` for the models of this package.

The viscous dissipation Phi = 2 eta (eps - tr(eps)/3 1) : eps of the
stream-function velocity, its (Di/Ra) source in the temperature equation,
the budget and the identity <Phi> = Ra <theta u_z> with its state-dependent
bound (``physics/dissipation.py:187-575``).  The fields run on the model's
transforms (:mod:`specmc_gb300.energy`); this module adds the source helpers,
the single-mode closed forms and the bound of the identity.
"""
from __future__ import annotations

import numpy as np

from .energy import phi_coeffs, phi_field, phi_integral, phi_padded, pi_theta, strain_fields
from .energy import dissipation_balance as balance

__all__ = ["PHI_FORM", "DI_DEFINITION", "COEFFICIENT", "ETA_CLASSES", "J9_2_TOL",
           "J9_2_TOL_GENERAL", "J9_2_TAIL_SLACK", "eta_class", "strain_fields", "phi_padded",
           "phi_coeffs", "phi_field", "phi_integral", "phi_z_tail", "j9_2_bound", "pi_theta",
           "source_coeffs", "source_integral", "add_dissipation_source",
           "single_mode_theta_integral", "single_mode_psi_integral", "nu_top_steady",
           "nu_bot_steady", "balance"]

PHI_FORM = "2 eta (eps - (1/3) tr(eps) 1) : eps"
DI_DEFINITION = "Di = alpha0 g0 d / cP0"
COEFFICIENT = "Di / Ra"
ETA_CLASSES = ("const", "eta_z", "eta_xz")
#: bound of |<Phi> / (Ra <theta u_z>) - 1| per eta class, the reference's
#: measured floor on a resolved state (physics/dissipation.py:196-207)
J9_2_TOL = {"const": 1e-14, "eta_z": 1e-12, "eta_xz": 1e-9}
J9_2_TOL_GENERAL = 1e-9
#: fraction of Phi's own z-Chebyshev tail the identity may miss on an
#: under-resolved state (physics/dissipation.py:209-225)
J9_2_TAIL_SLACK = 0.05


def eta_class(eta):
    """'const' (None or uniform), 'eta_z' (a profile, or the same in every
    column) or 'eta_xz'."""
    if eta is None:
        return "const"
    e = np.asarray(eta, dtype=float)
    if e.ndim < 2 or e.size == 0:
        return "eta_z"
    if (e == e.flat[0]).all():
        return "const"
    return "eta_z" if (e == e[:1]).all() else "eta_xz"


def phi_z_tail(model, psi, eta=None, n_last=6):
    """Largest magnitude among the last ``n_last`` Chebyshev coefficients of
    Phi (tau rows kept), relative to its largest coefficient."""
    c = np.abs(phi_coeffs(model, psi, eta, tau_zero=False))
    return float(c[:, -int(n_last):].max() / max(float(c.max()), 1e-300))


def j9_2_bound(eta_cls="eta_xz", tau_S=0.0, phi_tail=0.0):
    """The identity's bound: the class floor, 10x the Stokes tolerance or the
    tail slack times Phi's z-tail, whichever is largest."""
    floor = J9_2_TOL.get(str(eta_cls), J9_2_TOL_GENERAL)
    return max(floor, 10.0 * float(tau_S), J9_2_TAIL_SLACK * float(phi_tail))


def source_coeffs(model, psi, eta=None, Di=0.0, Ra=None, tau_zero=True):
    """-> (Di/Ra) Phi as (Nk, Nz) coefficients; zeros (without evaluating Phi)
    when Di == 0."""
    out = np.zeros((int(model.Nk), int(model.Nz)), dtype=complex)
    if float(Di) == 0.0:
        return out
    ra = float(model.Ra if Ra is None else Ra)
    if not (np.isfinite(ra) and ra > 0.0):
        raise ValueError("the (Di/Ra) source needs a finite Ra > 0, have %r" % (ra,))
    return out + (float(Di) / ra) * phi_coeffs(model, psi, eta, tau_zero=tau_zero)


def source_integral(model, coeffs):
    """The volume mean of a coefficient field, by the model's own quadrature."""
    return float(model.vol_mean(model.grid(np.asarray(coeffs))))


def add_dissipation_source(b, coeffs, Di):
    """-> the raveled right-hand side ``b`` plus ``coeffs`` on the equation
    rows (the two tau rows untouched); the same object when Di == 0."""
    if float(Di) == 0.0:
        return b
    c = np.asarray(coeffs)
    out = np.array(b, dtype=complex).reshape(c.shape)
    out[:, :-2] += c[:, :-2]
    return out.ravel()


def single_mode_theta_integral(Ra, kx, kz, amp):
    """<Phi> of the Stokes flow driven by theta = amp cos(kx x) sin(kz z) at
    eta = 1: Ra^2 kx^2 amp^2 / (4 g^2), g = kx^2 + kz^2."""
    g = float(kx) ** 2 + float(kz) ** 2
    return (float(Ra) * float(kx) * float(amp)) ** 2 / (4.0 * g * g)


def single_mode_psi_integral(kx, kz, A):
    """<Phi> of psi = A sin(kx x) sin(kz z) at eta = 1: A^2 g^2 / 4."""
    g = float(kx) ** 2 + float(kz) ** 2
    return float(A) ** 2 * g * g / 4.0


def nu_top_steady(uz_theta, H=0.0, phi_total=0.0):
    """Nu_top at a steady state with both sources: 1 + <u_z theta> + H/2 + <S_Phi>/2."""
    return 1.0 + float(uz_theta) + 0.5 * (float(H) + float(phi_total))


def nu_bot_steady(uz_theta, H=0.0, phi_total=0.0):
    """Nu_bot at the same state: 1 + <u_z theta> - H/2 - <S_Phi>/2."""
    return 1.0 + float(uz_theta) - 0.5 * (float(H) + float(phi_total))
