"""The TALA route (compressibility='tala') on the GPU, through the C ABI,
against fixtures the reference wrote (tests/golden/tala_ops_16x12.npz,
march_tala_*.npz) and the oracle.

TALA changes the velocity on every model (u = curl(Psi) / rho_bar), the
temperature equation of the eta_z / eta_T models (rho_bar weights, rho_bar H,
the adiabatic source, the rho_bar preconditioner) and the coupled Stokes
operator of the eta_T model (L^(rho) Green functions, the distributed-form
A12 block, the rho_bar^2 buoyancy, omega = -v / rho_bar).  Tolerances are
those of the Boussinesq parity tests: FP64 with a different arithmetic order,
states to roundoff amplified by the conditioning (1e-11 isoviscous, 1e-9
eta_z, 1e-7 coupled whose Stokes solve converges to 1e-8), Nu and Vrms far
inside the 1e-6 bar.
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def gb():
    from specmc_gb300 import _lib
    _lib.build()
    import specmc_gb300.api as api
    from specmc_gb300.config import ConvectionConfig
    return api, ConvectionConfig, _lib


def _matvec(m, lib, eta, v):
    out = np.empty_like(v)
    e = np.ascontiguousarray(eta)
    lib.check(m._lib.smc_schur_matvec(m._h, e.ctypes.data_as(ctypes.c_void_p),
                                      v.ctypes.data_as(ctypes.c_void_p),
                                      out.ctypes.data_as(ctypes.c_void_p), 0))
    return out.ravel()


def test_tala_operators_match_reference(gb):
    """eta, the matrix-free TALA Schur action (pseudo-spectral and dense
    product forms), the Stokes solve, the velocity and one step."""
    from oracle import specmc_oracle as O
    api, CC, lib = gb
    g = _load("tala_ops_16x12.npz")
    cfg = CC(Ra=1e4, Nx=16, Nz=12, viscosity_model="eta_T", compressibility="tala",
             dissipation_number=0.7, precond="legacy")
    m = api.build_model(cfg)
    assert m.tala_active and m.tala_a == g["tala_a"].item()
    # a host-side exp: the libm of the machine that wrote the fixture may
    # round the last bit differently
    np.testing.assert_allclose(m.rho_grid, g["rho_grid"], rtol=4.5e-16, atol=0.0)
    assert _rel(m.rho_c, g["rho_c"]) < 1e-15 and _rel(m.rho2_c, g["rho2_c"]) < 1e-15
    eta = m.eta_of(g["that"])
    assert _rel(eta, g["eta"]) < 1e-13
    v = np.ascontiguousarray(g["v"].reshape(m.Nk, m.Nz))
    assert _rel(_matvec(m, lib, g["eta"], v), g["Av"]) < 1e-12
    lib.check(m._lib.smc_set_option(m._h, b"dense_mult_eta", 1.0))
    assert _rel(_matvec(m, lib, g["eta"], v), g["Av"]) < 1e-12
    o = O.build(cfg)
    m2 = api.build_model(cfg)
    psi, om = m2.stokes(g["that"])
    psi_o, om_o = o.stokes(g["that"])
    assert _rel(psi, psi_o) < 1e-8 and _rel(om, om_o) < 1e-8
    ux, uz = m2.velocity(psi_o)
    ux_o, uz_o = o.velocity(psi_o)
    assert _rel(ux, ux_o) < 1e-12 and _rel(uz, uz_o) < 1e-12
    m3 = api.build_model(cfg)
    assert _rel(m3.step(g["that"], g["dt"].item()), g["that1"]) < 1e-8


CASES = [
    ("tala_const_32x24", 1e-11, 1e-11),
    ("tala_etaz_32x24", 1e-9, 1e-10),
    ("tala_etaT_32x24", 1e-7, 1e-8),
    ("tala_arrhenius_32x24", 1e-7, 1e-8),
]


@pytest.mark.parametrize("case,state_tol,diag_tol", CASES)
def test_tala_march_matches_reference(gb, case, state_tol, diag_tol):
    api, CC, lib = gb
    g = _load("march_%s.npz" % case)
    m = api.build_model(CC(**{k[4:]: g[k].item() for k in g.files if k.startswith("cfg_")}))
    s = np.array(g["that0"], copy=True)
    worst = 0.0
    for n in range(len(g["dts"])):
        dt = api.production_dt(m, s)
        assert abs(dt - g["dts"][n]) <= 1e-9 * g["dts"][n], (n, dt, g["dts"][n])
        s = m.step(s, dt)
        worst = max(worst, _rel(s, g["states"][n]))
    assert worst < state_tol, worst
    d = m.diagnostics(s)
    for key in ("Nu_top", "Nu_bot", "Nu_energy", "urms", "umax", "amp"):
        ref = g["diag_" + key].item()
        assert abs(d[key] - ref) <= diag_tol * max(abs(ref), 1e-300), (key, d[key], ref)
    c = m.counters()
    for key in ("n_refresh", "n_defect", "n_defect_failed", "n_defect_double_fail", "n_steps"):
        if "ctr_" + key in g.files:
            assert c[key] == int(g["ctr_" + key]), (key, c[key], int(g["ctr_" + key]))


@pytest.mark.parametrize("vm,kw", [("eta_z", dict(deta_T=100.0)), ("eta_T", dict(precond="legacy"))])
def test_tala_at_zero_Di_is_boussinesq(gb, vm, kw):
    """With Di = 0 (rho_bar = 1, a = 0) the TALA kernels reproduce the
    Boussinesq route (the limit stokes_tala.py:523-548 checks): six steps of
    both on the GPU agree to roundoff (3e-15 on the oracle)."""
    api, CC, lib = gb
    mb = api.build_model(CC(Ra=1e4, Nx=32, Nz=24, viscosity_model=vm, **kw))
    mt = api.build_model(CC(Ra=1e4, Nx=32, Nz=24, viscosity_model=vm, compressibility="tala", **kw))
    sb = mb.seed(amp=3e-2, m=1, n=1)
    st = np.array(sb, copy=True)
    for _ in range(6):
        sb = mb.step(sb, api.production_dt(mb, sb))
        st = mt.step(st, api.production_dt(mt, st))
    assert _rel(st, sb) < 1e-9, _rel(st, sb)
