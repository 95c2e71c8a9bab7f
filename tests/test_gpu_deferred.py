"""The march's deferred work: inside smc_advance / smc_march_adaptive the
engine results are read at the next synchronisation the step needs anyway,
the step's mirror projections and Stokes-memo test travel with the CFL
reduction, the viscosity counters accumulate on the device and the BFBT
blocks' reuse is decided on the device.  None of that may change a number:
the resident march, the one-call march and the stepwise host loop (which
synchronises after every solve) give the same bits and the same counters."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 30
KEYS = ("n_steps", "n_stokes", "n_memo_hits", "n_bfbt_solves", "n_bfbt_iters", "n_bfbt_rescue",
        "n_clip_T", "n_T_out_of_range", "n_clip_eta", "n_smooth_eta", "n_clip_eta_proj",
        "n_smooth_eta_proj", "n_theta_nonconv", "n_theta_solves", "n_theta_iters",
        "theta_last_iters", "max_T_excursion", "theta_last_res", "last_bfbt_true_res")


@pytest.fixture(scope="module")
def gb():
    from specmc_gb300 import _lib
    _lib.build()
    import specmc_gb300.api as api
    from specmc_gb300.config import ConvectionConfig
    return api, ConvectionConfig, _lib


def _resident(api, lib, cfg, th0):
    m = api.build_model(cfg, form="mixed")
    s = np.ascontiguousarray(th0)
    lib.check(m._lib.smc_set_state(m._h, s.ctypes.data_as(ctypes.c_void_p), lib.SMC_HOST))
    info = lib.SmcMarchInfo()
    t = 0.0
    for _ in range(STEPS):
        lib.check(m._lib.smc_advance(m._h, 1e30, 1, 40.0, 4e-5, ctypes.byref(info)))
        t = info.t
    out = np.empty_like(s)
    lib.check(m._lib.smc_get_state(m._h, out.ctypes.data_as(ctypes.c_void_p), lib.SMC_HOST))
    c = m.counters()
    m.close()
    return out, c, t


@pytest.mark.parametrize("Nx,Nz,deta", [(64, 96, 1000.0), (32, 24, 1e4)])
def test_deferred_march_equals_stepwise(gb, Nx, Nz, deta):
    api, CC, lib = gb
    cfg = CC(viscosity_model="eta_T", deta_T=deta, Ra=1e4, Nx=Nx, Nz=Nz)
    m0 = api.build_model(cfg, form="mixed")
    th0 = m0.seed(amp=3e-2, m=1, n=1)
    m0.close()
    sa, ca, t_end = _resident(api, lib, cfg, th0)
    # the one-call march over the same steps
    mb = api.build_model(cfg, form="mixed")
    sb, info = mb.march_adaptive(th0, 1e30, safety=40.0, dtmax=4e-5, max_steps=STEPS)
    cb = mb.counters()
    mb.close()
    assert info["steps"] == STEPS and info["t"] == t_end
    # the stepwise host loop: every solve synchronised, nothing prefetched
    mc = api.build_model(cfg, form="mixed")
    sc = np.array(th0, copy=True)
    for _ in range(STEPS):
        sc = mc.step(sc, mc.production_dt(sc, safety=40.0, dtmax=4e-5))
    cc = mc.counters()
    mc.close()
    assert np.array_equal(sa, sc) and np.array_equal(sb, sc)
    for key in KEYS:
        assert ca[key] == cc[key] == cb[key], (key, ca[key], cb[key], cc[key])
    assert ca["n_stokes"] >= STEPS and ca["n_theta_solves"] == STEPS


def test_deferred_failed_solves_equal_stepwise(gb):
    """The same comparison when every BFBT solve fails (a one-iteration
    budget): the deferred Stokes result is read after the CFL reduction and
    turns into the FP64 fallback and the dense rescue there, and what was
    computed from the failed solve (psi, omega, the velocity, the CFL
    reduction) is computed again; the later solves take the lagged-factor
    route.  The resident march and the stepwise host loop give the same bits
    and counters."""
    from specmc_gb300.solver import RBCCoupled
    api, CC, lib = gb
    kw = dict(Nx=32, Nz=24, deta_T=1000.0, stokes_maxiter=1, form="mixed")
    m0 = RBCCoupled(**kw)
    th0 = np.ascontiguousarray(m0.seed(amp=3e-2, m=1, n=1))
    m0.close()
    steps = 12
    ma = RBCCoupled(**kw)
    _lib = ma._lib
    lib.check(_lib.smc_set_state(ma._h, th0.ctypes.data_as(ctypes.c_void_p), lib.SMC_HOST))
    info = lib.SmcMarchInfo()
    for _ in range(steps):
        lib.check(_lib.smc_advance(ma._h, 1e30, 1, 40.0, 4e-5, ctypes.byref(info)))
    sa = np.empty_like(th0)
    lib.check(_lib.smc_get_state(ma._h, sa.ctypes.data_as(ctypes.c_void_p), lib.SMC_HOST))
    ca = ma.counters()
    ma.close()
    mc = RBCCoupled(**kw)
    sc = np.array(th0, copy=True)
    for _ in range(steps):
        sc = mc.step(sc, mc.production_dt(sc, safety=40.0, dtmax=4e-5))
    cc = mc.counters()
    mc.close()
    assert ca["n_bfbt_rescue"] >= 1
    assert np.array_equal(sa, sc)
    for key in KEYS + ("n_refresh", "n_defect"):
        assert ca[key] == cc[key], (key, ca[key], cc[key])
