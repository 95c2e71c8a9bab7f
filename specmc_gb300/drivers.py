"""Model-level drivers of the reference's model classes, for any model with
the reference's contract.

* ``run(model, that, tstop, ...)``: the simple CFL march of
  ``specmc/core/rbc_galerkin.py:473-491`` (``RBC.run``): step until ``tstop``
  with a fixed ``dt`` or ``model.cfl_dt(that, safety, dtmax)``, recording the
  diagnostics (plus ``t`` and ``dt``) whenever the model's step counter is a
  multiple of ``cadence``; -> (state, records).
* ``mirror_error(model, that)``: max |theta(x) - theta(Lx - x)| / max |theta|
  on the model grid (``rbc_galerkin.py:455-463``); on the nodes x_j = j Lx/Nx
  the reflection is the index map j -> (-j) mod Nx.
"""
from __future__ import annotations

import numpy as np

__all__ = ["run", "mirror_error"]


def _host(a):
    return a.cpu().numpy() if hasattr(a, "cpu") else np.asarray(a)


def mirror_error(model, that):
    g = _host(model.grid(that))
    mirrored = g[(-np.arange(int(model.Nx))) % int(model.Nx), :]
    return float(np.abs(g - mirrored).max() / max(np.abs(g).max(), 1e-300))


def run(model, that, tstop, dt=None, safety=0.5, dtmax=5e-3, cadence=200, verbose=True):
    t, records = 0.0, []
    s = that
    while t < tstop:
        step_dt = dt if dt is not None else model.cfl_dt(s, safety, dtmax)
        s = model.step(s, step_dt)
        t += step_dt
        if int(model.n_steps) % cadence == 0:
            rec = dict(model.diagnostics(s), t=t, dt=step_dt)
            records.append(rec)
            if verbose:
                print("  t=%8.4f Nu=%9.5f/%9.5f urms=%8.4f umax=%8.3f amp=%.3e dt=%.2e"
                      % (t, rec["Nu_top"], rec["Nu_bot"], rec["urms"], rec["umax"], rec["amp"],
                         step_dt), flush=True)
    return s, records
