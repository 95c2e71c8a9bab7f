"""The temperature- and depth-dependent viscosity laws on the host
(``specmc/physics/viscosity.py:157-194``): the exponential law of
Blankenbach case 2a, eta(T) = exp(-ln(deta_T) T), its value on the
conductive profile T = 1 - z (the frozen depth-only viscosity) and the
depth-law switch of the depth-only model.  The GPU evaluates the same laws
in its eta kernels; these are for drivers and checks."""
from __future__ import annotations

import numpy as np

__all__ = ["eta_exp_T", "eta_conductive_background", "eta_from_law"]


def eta_exp_T(T, deta_T):
    """exp(-ln(deta_T) T)."""
    return np.exp(-np.log(float(deta_T)) * np.asarray(T, dtype=float))


def eta_conductive_background(z, deta_T, Tbot=1.0, Ttop=0.0):
    """The exponential law on the linear profile T = Tbot + (Ttop - Tbot) z
    (weak at the hot bottom z = 0, eta = 1 at the cold top)."""
    return eta_exp_T(Tbot + (Ttop - Tbot) * np.asarray(z, dtype=float), deta_T)


def eta_from_law(law, deta_T, z):
    """The depth-only viscosity of ``law``: ones for 'isoviscous' (aliases
    'const', 'constant'), the conductive background for 'exp_T_depth'
    (alias 'depth_exp'); NotImplementedError for any other name."""
    key = str(law).lower()
    if key in ("isoviscous", "const", "constant"):
        return np.ones_like(np.asarray(z, dtype=float))
    if key in ("exp_t_depth", "depth_exp"):
        return eta_conductive_background(z, deta_T)
    raise NotImplementedError("viscosity_law %r: the depth-only laws are 'isoviscous' and "
                              "'exp_T_depth'" % (law,))
