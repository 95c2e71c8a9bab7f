"""The depth-only scenario (``viscosity_model='eta_z'``), as
``specmc/models/eta_z.py:32-59``: frozen eta(z) Stokes + BDF2 theta."""
from __future__ import annotations

from .. import _numerics as NUM
from ..solver import RBCImplicitTheta

__all__ = ["NAME", "CLS", "BUILDER", "kwargs", "build", "spec"]

NAME = "eta_z"
CLS = RBCImplicitTheta
BUILDER = "make_convection"


def kwargs(cfg):
    return dict(Ra=cfg.Ra, Nx=int(cfg.Nx), Nz=int(cfg.Nz), Lx=cfg.Lx,
                viscosity_law="exp_T_depth", deta_T=float(cfg.deta_T),
                symmetrize=bool(cfg.symmetrize), zform=NUM.ZFORM,
                theta_scheme=NUM.THETA_SCHEME, implicit_buoy=NUM.IMPLICIT_BUOY,
                theta_rtol=NUM.THETA_RTOL, theta_extrapolate=NUM.THETA_EXTRAPOLATE,
                internal_heating=float(cfg.internal_heating),
                dissipation_number=float(cfg.dissipation_number),
                compressibility=str(cfg.compressibility),
                eta_min=float(cfg.eta_min), eta_max=float(cfg.eta_max),
                eta_smooth=float(cfg.eta_smooth))


def build(**kw):
    return RBCImplicitTheta(**kw)


def spec(cfg, compressibility):
    return dict(model=NAME, compressibility=compressibility, builder=BUILDER,
                cls=CLS, kwargs=kwargs(cfg))
