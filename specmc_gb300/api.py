"""Public API: ConvectionConfig -> GPU model -> march.

The drop-in twin of ``specmc/api.py``: the same functions, argument meanings
and dispatch table (``MODEL_MODULES``), building the GPU models of
:mod:`specmc_gb300.solver`.  ``march_adaptive`` keeps the state on the GPU
between steps (one native call for the whole march).
"""
from __future__ import annotations

import numpy as np

from . import _numerics as NUM
from .config import (ConvectionConfig, normalize_compressibility,
                     normalize_viscosity_model)
from .recipes import const as _model_const
from .recipes import eta_T as _model_eta_T
from .recipes import eta_z as _model_eta_z

__all__ = ["MODEL_MODULES", "MODEL_CLASSES", "numerics", "model_spec", "model_kwargs",
           "build_model", "describe", "production_dt", "load_checkpoint", "march",
           "march_adaptive"]

#: viscosity_model -> recipe module (specmc/api.py:53-58)
MODEL_MODULES = {
    "const": _model_const,
    "eta_z": _model_eta_z,
    "eta_T": _model_eta_T,
    "arrhenius": _model_eta_T,
}
MODEL_CLASSES = {name: mod.CLS for name, mod in MODEL_MODULES.items()}


def numerics():
    """The fixed internal numerical constants (a copy)."""
    return NUM.as_dict()


def model_spec(cfg: ConvectionConfig):
    """The construction recipe for ``cfg`` (specmc/api.py:73-94)."""
    if not isinstance(cfg, ConvectionConfig):
        raise TypeError("expected ConvectionConfig, got %r" % (type(cfg),))
    cfg.validate()
    vm = normalize_viscosity_model(cfg.viscosity_model)
    comp = normalize_compressibility(cfg.compressibility)
    module = MODEL_MODULES.get(vm)
    if module is None:
        raise NotImplementedError("viscosity_model=%r is not implemented" % (vm,))
    return module.spec(cfg, comp)


def model_kwargs(cfg: ConvectionConfig):
    return dict(model_spec(cfg)["kwargs"])


def build_model(cfg: ConvectionConfig, form="plain", device=0):
    """Build the GPU model for ``cfg`` and check its class (specmc/api.py:102-110).

    ``form='plain'`` (default) is the FP64 GPU port of the reference algorithm,
    route for route.  ``form='mixed'`` is the fast form: the coupled Stokes
    system is solved by spectral-BFBT preconditioned FGMRES (FP64 outer loop
    and residuals) whatever ``cfg.precond`` says, with the per-wavenumber block
    preconditioners applied as explicit FP64 inverse operators; it agrees with
    the plain form to the solver tolerances (1e-8 Stokes, 1e-10 theta).
    ``compressibility='tala'`` runs the plain form only (the mixed form's
    block preconditioner is the Boussinesq BFBT model, which the reference
    has no TALA form of): ``form='mixed'`` raises NotImplementedError.
    """
    spec = model_spec(cfg)
    model = MODEL_MODULES[spec["model"]].build(**spec["kwargs"], form=form, device=device)
    if type(model) is not spec["cls"]:
        raise AssertionError("internal mapping error: viscosity_model=%r built %s, expected %s"
                             % (spec["model"], type(model).__name__, spec["cls"].__name__))
    return model


def describe(cfg: ConvectionConfig):
    """A JSON-safe description of what ``cfg`` will run (specmc/api.py:113-120)."""
    spec = model_spec(cfg)
    return dict(config=cfg.canonical(), model=spec["model"],
                model_class=spec["cls"].__name__, builder=spec["builder"],
                ctor_kwargs={k: (None if v is None else v) for k, v in spec["kwargs"].items()},
                numerics=numerics())


def production_dt(model, that):
    """dt = min(DTMAX, CFL_SAFETY x CFL) (specmc/api.py:126-133)."""
    return float(model.production_dt(that, safety=NUM.CFL_SAFETY, dtmax=NUM.DTMAX))


def load_checkpoint(path):
    """(theta coefficients, meta) from a driver checkpoint .npz; delegates to
    :func:`specmc_gb300.checkpoint.load` (specmc/api.py -> io/checkpoint.py:80-103)."""
    from . import checkpoint
    return checkpoint.load(path)


def march(model, that, dt, nsteps, keep_states=False, on_step=None):
    """Fixed-dt march (specmc/api.py:147-166)."""
    dt = float(dt)
    nsteps = int(nsteps)
    if not keep_states and on_step is None:
        s = model.march(that, dt, nsteps)
        return s, dict(steps=nsteps, t=nsteps * dt, dt=dt)
    s = np.array(that, copy=True) if not hasattr(that, "is_cuda") else that.clone()
    states = [] if keep_states else None
    for n in range(nsteps):
        s = model.step(s, dt)
        if states is not None:
            states.append(s)
        if on_step is not None:
            on_step(n + 1, (n + 1) * dt, s)
    info = dict(steps=nsteps, t=nsteps * dt, dt=dt)
    if states is not None:
        info["states"] = np.array([np.asarray(x) for x in states])
    return s, info


def march_adaptive(model, that, tstop, safety=None, dtmax=None, on_step=None):
    """CFL-limited march to ``tstop`` (specmc/api.py:169-190).

    Without ``on_step`` the whole loop runs inside one native call and the
    state stays on the GPU; with it, each step returns to Python.
    """
    safety = NUM.CFL_SAFETY if safety is None else float(safety)
    dtmax = NUM.DTMAX if dtmax is None else float(dtmax)
    if on_step is None:
        s, info = model.march_adaptive(that, float(tstop), safety=safety, dtmax=dtmax)
        info.update(safety=safety, dtmax=dtmax)
        return s, info
    s = np.array(that, copy=True) if not hasattr(that, "is_cuda") else that.clone()
    t, n, dt = 0.0, 0, float("nan")
    while t < float(tstop):
        dt = float(model.production_dt(s, safety=safety, dtmax=dtmax))
        s = model.step(s, dt)
        t += dt
        n += 1
        on_step(n, t, s)
    return s, dict(steps=n, t=t, dt=dt, safety=safety, dtmax=dtmax)
