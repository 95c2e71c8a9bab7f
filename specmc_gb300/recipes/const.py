"""The isoviscous scenario (``viscosity_model='const'``), as
``specmc/models/const.py:37-57``: the explicit-advection RBC model."""
from __future__ import annotations

from ..solver import RBC

__all__ = ["NAME", "CLS", "BUILDER", "kwargs", "build", "spec"]

NAME = "const"
CLS = RBC
BUILDER = "make_convection"


def kwargs(cfg):
    return dict(Ra=cfg.Ra, Nx=int(cfg.Nx), Nz=int(cfg.Nz), Lx=cfg.Lx,
                viscosity_law="isoviscous", deta_T=float(cfg.deta_T),
                internal_heating=float(cfg.internal_heating),
                dissipation_number=float(cfg.dissipation_number),
                compressibility=str(cfg.compressibility))


def build(**kw):
    return RBC(**kw)


def spec(cfg, compressibility):
    return dict(model=NAME, compressibility=compressibility, builder=BUILDER,
                cls=CLS, kwargs=kwargs(cfg))
