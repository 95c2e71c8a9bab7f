"""The temperature-dependent scenarios (``'eta_T'`` and ``'arrhenius'``), as
``specmc/models/eta_T.py:44-102``: the coupled model."""
from __future__ import annotations

from .. import _numerics as NUM
from ..solver import RBCCoupled

__all__ = ["NAME", "CLS", "BUILDER", "kwargs", "build", "spec"]

NAME = "eta_T"
CLS = RBCCoupled
BUILDER = "RBCCoupled"


def kwargs(cfg):
    dtol = float(cfg.defect_tol)
    return dict(Ra=cfg.Ra, Nx=int(cfg.Nx), Nz=int(cfg.Nz), Lx=cfg.Lx,
                deta_T=float(cfg.deta_T), symmetrize=bool(cfg.symmetrize),
                zform=NUM.ZFORM, theta_scheme=NUM.THETA_SCHEME,
                theta_extrapolate=NUM.THETA_EXTRAPOLATE,
                implicit_buoy=NUM.IMPLICIT_BUOY, stokes_mode=NUM.STOKES_MODE,
                lag=int(cfg.lag), K=int(cfg.K), stokes_rtol=NUM.STOKES_RTOL,
                defect_tol=(None if dtol <= 0.0 else dtol), max_K=int(cfg.max_K),
                eta_drift_tol=NUM.ETA_DRIFT_TOL, eta_dealias=NUM.ETA_DEALIAS,
                internal_heating=float(cfg.internal_heating),
                dissipation_number=float(cfg.dissipation_number),
                compressibility=str(cfg.compressibility),
                arrhenius_Ts=float(cfg.arrhenius_Ts),
                arrhenius_E=float(cfg.arrhenius_E),
                arrhenius_V=float(cfg.arrhenius_V),
                reference_anchor=str(cfg.reference_anchor),
                eta_min=float(cfg.eta_min), eta_max=float(cfg.eta_max),
                eta_smooth=float(cfg.eta_smooth),
                precond=str(cfg.precond).strip().lower())


def build(**kw):
    return RBCCoupled(**kw)


def spec(cfg, compressibility):
    return dict(model=NAME, compressibility=compressibility, builder=BUILDER,
                cls=CLS, kwargs=kwargs(cfg))
