"""The model-level drivers (specmc_gb300.drivers: RBC.run and
RBC.mirror_error of core/rbc_galerkin.py:455-491) against records the
reference wrote (tests/golden/drivers_32x24.npz).  They take any model with
the reference's contract; the oracle's isoviscous model stands in for the GPU
one here (the GPU models delegate their run / mirror_error methods to
these functions)."""
import os

import numpy as np

from oracle import specmc_oracle as O

from conftest import GOLDEN


def test_run_and_mirror_error_match_reference():
    from specmc_gb300 import drivers
    g = np.load(os.path.join(GOLDEN, "drivers_32x24.npz"))
    m = O.ConstModel(Ra=1e4, Nx=32, Nz=24)
    s, hist = drivers.run(m, g["that0"], tstop=30 * 4e-5 * 0.999, safety=0.5, dtmax=4e-5,
                          cadence=10, verbose=False)
    assert m.n_steps == int(g["n_steps"])
    keys = [str(k) for k in g["keys"]]
    assert len(hist) == len(g["hist"]) and sorted(hist[0]) == keys
    got = np.array([[h[k] for k in keys] for h in hist])
    assert np.abs(got - g["hist"]).max() <= 1e-12 * np.abs(g["hist"]).max()
    assert np.abs(s - g["final"]).max() <= 1e-12 * np.abs(g["final"]).max()
    assert drivers.mirror_error(m, s) < 1e-14
    assert abs(drivers.mirror_error(m, g["odd"]) - g["mirror_odd"].item()) <= 1e-14


def test_theta_solver_view_names():
    """model.theta maps the reference's ImplicitThetaSolver names onto the
    model's counters and configuration (a stand-in model supplies both)."""
    from types import SimpleNamespace
    from specmc_gb300.solver import ThetaSolverView
    counters = dict(theta_last_iters=7, theta_last_res=3e-11, n_theta_nonconv=1,
                    n_be_fallback=2, n_theta_solves=9)
    model = SimpleNamespace(counters=lambda: counters, internal_heating=1.5, dissipation_number=0.25,
                            _cfg=SimpleNamespace(theta_rtol=1e-10, theta_restart=40, theta_maxiter=200))
    t = ThetaSolverView(model)
    assert (t.last_iters, t.last_res, t.n_nonconv, t.n_be_fallback, t.n_solves) == (7, 3e-11, 1, 2, 9)
    assert (t.scheme, t.rtol, t.restart, t.maxiter) == ("bdf2", 1e-10, 40, 200)
    assert (t.internal_heating, t.dissipation_number) == (1.5, 0.25)
