"""``specmc.physics.heating`` for the models of this package.

Constant internal heating H: its exact conductive state
(``physics/heating.py:168-199``), its spectral source (one coefficient, the
T_0 term of the k = 0 mode, ``:204-240``), the steady energy identities
(``:245-253``), and the budgets of a state, which run on the model's
transforms (:func:`specmc_gb300.energy.heating_balance` as ``balance``,
``flux_profile``).
"""
from __future__ import annotations

import numpy as np

from .energy import flux_profile, nu_pair, theta_mean
from .energy import heating_balance as balance
from .initial import heated_conductive_theta as conductive_theta

__all__ = ["conductive_theta", "conductive_T", "mean_T_conductive", "nu_bot_conductive",
           "nu_top_conductive", "T_max_conductive", "source_coeffs", "add_constant_source",
           "source_integral", "nu_energy_steady", "nu_bot_energy_steady", "balance",
           "flux_profile", "nu_pair", "theta_mean"]


def conductive_T(z, H):
    """T(z) = (1 - z) + H z (1 - z) / 2 of the motionless heated state."""
    return (1.0 - np.asarray(z, dtype=float)) + conductive_theta(z, H)


def mean_T_conductive(H):
    """<T> of the conductive state, 1/2 + H/12."""
    return 0.5 + float(H) / 12.0


def nu_bot_conductive(H):
    """The bottom heat flux of the conductive state, 1 - H/2."""
    return 1.0 - float(H) / 2.0


def nu_top_conductive(H):
    """The top heat flux of the conductive state, 1 + H/2."""
    return 1.0 + float(H) / 2.0


def T_max_conductive(H):
    """-> (T_max, z_max): at the bottom wall (1, 0) for H <= 2, else the
    interior maximum at z = 1/2 - 1/H, T = 1/2 + H/8 + 1/(2H)."""
    H = float(H)
    if H <= 2.0:
        return 1.0, 0.0
    return 0.5 + H / 8.0 + 0.5 / H, 0.5 - 1.0 / H


def source_coeffs(Nk, Nz, H):
    """-> the (Nk, Nz) coefficients of theta_t += H: H on (k = 0, T_0) only."""
    out = np.zeros((int(Nk), int(Nz)), dtype=complex)
    out[0, 0] = float(H)
    return out


def add_constant_source(b, Nk, Nz, H):
    """-> the raveled right-hand side ``b`` with H added on (k = 0, T_0); the
    same object when H == 0."""
    if float(H) == 0.0:
        return b
    out = np.array(b, dtype=complex).reshape(int(Nk), int(Nz))
    out[0, 0] += float(H)
    return out.ravel()


def source_integral(H):
    """The volume integral of the source over the unit box: H."""
    return float(H)


def nu_energy_steady(uz_theta, H=0.0):
    """1 + <u_z theta>: at a steady state Nu_bot + H/2 = Nu_top - H/2 = this."""
    return 1.0 + float(uz_theta)


def nu_bot_energy_steady(uz_theta, H=0.0):
    """Nu_bot at a steady state, 1 + <u_z theta> - H/2."""
    return nu_energy_steady(uz_theta) - 0.5 * float(H)
