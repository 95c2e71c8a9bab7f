"""GPU path (through the C ABI) against the reference fixtures and the oracle.

Tolerances: the GPU path is FP64 with the reference's algorithm; its
arithmetic order differs from NumPy/LAPACK, so states agree to roundoff
amplified by the operator conditioning (~1e-12 relative per step measured on
the isoviscous case, ~1e-9 on the coupled cases whose Stokes solve is itself
only converged to 1e-8).  Nu and Vrms -- the reported quantities -- must agree
to 1e-6 relative (the bar stated for this path); the tests demand more where
the algorithm allows it.
"""
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
    return api, ConvectionConfig


def _cfg_kw(g):
    return {k[4:]: g[k].item() for k in g.files if k.startswith("cfg_")}


def test_transforms_match_reference(gb):
    api, CC = gb
    g = _load("transforms_16x12.npz")
    m = api.build_model(CC(viscosity_model="const", Nx=16, Nz=12))
    assert _rel(m.grid(g["cf"]), g["grid"]) < 1e-13
    assert _rel(m.coeffs(g["g"]), g["coeffs"]) < 1e-13
    assert _rel(m._synth_pad(g["cf"]), g["synth_pad"]) < 1e-13
    assert _rel(m._trunc_pad(g["gp"]), g["trunc_pad"]) < 1e-13
    psi, om = m.stokes(g["cf"])
    assert _rel(psi, g["psi"]) < 1e-12 and _rel(om, g["om"]) < 1e-12
    ux, uz = m.velocity(psi)
    assert _rel(ux, g["ux"]) < 1e-12 and _rel(uz, g["uz"]) < 1e-12
    assert _rel(m.step(g["cf"], 1e-4), g["step"]) < 1e-12
    assert _rel(m.seed(amp=3e-2, m=1, n=1), g["seed"]) < 1e-14


def test_coupled_operator_matches_reference(gb):
    api, CC = gb
    g = _load("coupled_ops_16x12.npz")
    m = api.build_model(CC(viscosity_model="eta_T", Nx=16, Nz=12))
    import ctypes
    from specmc_gb300 import _lib
    eta = np.empty((16, 12))
    th = np.ascontiguousarray(g["that"], dtype=np.complex128)
    _lib.check(m._lib.smc_eta_of(m._h, th.ctypes.data_as(ctypes.c_void_p), 0,
                                 eta.ctypes.data_as(ctypes.c_void_p)))
    assert _rel(eta, g["eta"]) < 1e-13
    v = np.ascontiguousarray(g["v"].reshape(m.Nk, m.Nz))
    out = np.empty_like(v)
    e = np.ascontiguousarray(g["eta"])
    _lib.check(m._lib.smc_schur_matvec(m._h, e.ctypes.data_as(ctypes.c_void_p),
                                       v.ctypes.data_as(ctypes.c_void_p),
                                       out.ctypes.data_as(ctypes.c_void_p), 0))
    assert _rel(out.ravel(), g["Av"]) < 1e-12
    m2 = api.build_model(CC(viscosity_model="eta_T", Nx=16, Nz=12))
    psi, om = m2.stokes(g["that"])
    assert _rel(psi, g["psi"]) < 1e-8 and _rel(om, g["om"]) < 1e-8


CASES = [
    ("const_32x24", 1e-11, 1e-11),
    ("etaz_32x24", 1e-9, 1e-10),
    ("etaT_32x24", 1e-7, 1e-8),
    ("etaT_bfbt_32x24", 1e-7, 1e-8),
    ("heated_2to1_32x24", 1e-7, 1e-8),
    ("arrhenius_32x24", 1e-7, 1e-8),
    ("smooth_32x24", 1e-7, 1e-8),
    ("arrhenius_pv_32x24", 1e-7, 1e-8),
]

EXACT_COUNTERS = ("n_refresh", "n_defect", "n_defect_failed", "n_defect_double_fail",
                  "n_bfbt_solves", "n_bfbt_rescue", "n_steps")


@pytest.mark.parametrize("case,state_tol,diag_tol", CASES)
def test_march_matches_reference(gb, case, state_tol, diag_tol):
    api, CC = gb
    g = _load("march_%s.npz" % case)
    m = api.build_model(CC(**_cfg_kw(g)))
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
    for key in EXACT_COUNTERS:
        if "ctr_" + key in g.files:
            assert c[key] == int(g["ctr_" + key]), (key, c[key], int(g["ctr_" + key]))
    if "ctr_theta_n_nonconv" in g.files:
        assert c["n_theta_nonconv"] == int(g["ctr_theta_n_nonconv"])
        assert c["n_be_fallback"] == int(g["ctr_theta_n_be_fallback"])
        assert abs(c["theta_last_iters"] - int(g["ctr_theta_last_iters"])) <= 2


def test_march_adaptive_on_device_matches_stepwise(gb):
    """api.march_adaptive (one native call) == the stepwise host loop."""
    api, CC = gb
    g = _load("march_const_32x24.npz")
    m = api.build_model(CC(**_cfg_kw(g)))
    s, info = api.march_adaptive(m, g["that0"], tstop=1e-3)
    assert info["steps"] == 25
    assert _rel(s, g["states"][-1]) < 1e-11
    d = m.diagnostics(s)
    assert abs(d["Nu_top"] - 1.0027843387) < 1e-9
    assert abs(d["urms"] - 6.7774209783) < 1e-8


def test_isoviscous_regression_target(gb):
    """The reference's frozen isoviscous regression target
    (specmc/physics/viscosity.py:150-151: Ra 1e4, 64x48, t = 0.25,
    Nu 4.885140, Vrms 42.872720), marched from the default seed (amp 1e-3)
    with the legacy CFL protocol it is stored under (safety 0.4, dtmax 5e-6,
    specmc/api.py:172-175), about 50 500 steps in one native call: Nu_top and
    urms to 1e-6 (the reference itself reproduces it to 4e-7 / 2e-8)."""
    api, CC = gb
    m = api.build_model(CC(viscosity_model="const", Ra=1e4, Nx=64, Nz=48))
    s, info = api.march_adaptive(m, m.seed(), tstop=0.25, safety=0.4, dtmax=5e-6)
    assert info["steps"] >= 50000 and info["t"] >= 0.25
    d = m.diagnostics(s)
    assert abs(d["Nu_top"] - 4.885140) <= 1e-6 * 4.885140, d["Nu_top"]
    assert abs(d["urms"] - 42.872720) <= 1e-6 * 42.872720, d["urms"]


def test_oracle_parity_64x96_coupled(gb):
    """The headline grid (eta_T 64x96): GPU vs the reference fixture."""
    api, CC = gb
    g = _load("march_etaT_64x96.npz")
    m = api.build_model(CC(**_cfg_kw(g)))
    s = np.array(g["that0"], copy=True)
    for n in range(len(g["dts"])):
        s = m.step(s, api.production_dt(m, s))
    assert _rel(s, g["states"][-1]) < 1e-7
    d = m.diagnostics(s)
    assert abs(d["Nu_top"] - g["diag_Nu_top"].item()) <= 1e-8 * abs(g["diag_Nu_top"].item())
    assert abs(d["urms"] - g["diag_urms"].item()) <= 1e-8 * abs(g["diag_urms"].item())


def test_pseudo_spectral_mult_eta_equals_dense(gb):
    """The default pseudo-spectral mult_eta evaluates the same linear map as the
    dense per-shift blocks of the reference (lagged_stokes.py:162-193)."""
    import ctypes
    from specmc_gb300 import _lib
    api, CC = gb
    rng = np.random.default_rng(5)
    cfg = CC(viscosity_model="eta_T", Nx=64, Nz=96)
    m_ps, m_dn = api.build_model(cfg), api.build_model(cfg)
    _lib.check(m_dn._lib.smc_set_option(m_dn._h, b"dense_mult_eta", 1.0))
    th = m_ps.seed(amp=0.3, m=1, n=1) + 0.05 * m_ps.seed(amp=1.0, m=3, n=2)
    eta = np.empty((64, 96))
    thc = np.ascontiguousarray(th)
    _lib.check(m_ps._lib.smc_eta_of(m_ps._h, thc.ctypes.data_as(ctypes.c_void_p), 0,
                                    eta.ctypes.data_as(ctypes.c_void_p)))
    v = np.ascontiguousarray(rng.standard_normal((m_ps.Nk, 96)) + 1j * rng.standard_normal((m_ps.Nk, 96)))
    outs = []
    for m in (m_ps, m_dn):
        o = np.empty_like(v)
        _lib.check(m._lib.smc_schur_matvec(m._h, eta.ctypes.data_as(ctypes.c_void_p),
                                           v.ctypes.data_as(ctypes.c_void_p),
                                           o.ctypes.data_as(ctypes.c_void_p), 0))
        outs.append(o)
    assert _rel(outs[0], outs[1]) < 1e-12


@pytest.mark.parametrize("case", ["etaT_32x24", "heated_2to1_32x24", "arrhenius_32x24",
                                  "arrhenius_pv_32x24"])
def test_mixed_form_matches_reference(gb, case):
    """The fast form reproduces the reference's Nu and Vrms to 1e-6 relative."""
    api, CC = gb
    g = _load("march_%s.npz" % case)
    m = api.build_model(CC(**_cfg_kw(g)), form="mixed")
    s = np.array(g["that0"], copy=True)
    for n in range(len(g["dts"])):
        dt = api.production_dt(m, s)
        assert abs(dt - g["dts"][n]) <= 1e-6 * g["dts"][n]
        s = m.step(s, dt)
    assert _rel(s, g["states"][-1]) < 1e-6
    d = m.diagnostics(s)
    for key in ("Nu_top", "urms", "Nu_energy"):
        ref = g["diag_" + key].item()
        assert abs(d[key] - ref) <= 1e-6 * abs(ref), (key, d[key], ref)


def test_fused_schur_matvec_variants(gb):
    """The fast form's fused FP64 operator equals the plain Schur matvec to
    roundoff; its FP32 inner-iteration operator to FP32 accuracy."""
    import ctypes
    from specmc_gb300 import _lib
    api, CC = gb
    rng = np.random.default_rng(9)
    cfg = CC(viscosity_model="eta_T", Nx=64, Nz=96)
    m = api.build_model(cfg, form="mixed")
    th = m.seed(amp=0.3, m=1, n=1) + 0.05 * m.seed(amp=1.0, m=3, n=2)
    eta = np.empty((64, 96))
    thc = np.ascontiguousarray(th)
    _lib.check(m._lib.smc_eta_of(m._h, thc.ctypes.data_as(ctypes.c_void_p), 0,
                                 eta.ctypes.data_as(ctypes.c_void_p)))
    v = np.ascontiguousarray(rng.standard_normal((m.Nk, 96)) + 1j * rng.standard_normal((m.Nk, 96)))
    outs = []
    for variant in (0, 1, 2):
        _lib.check(m._lib.smc_set_option(m._h, b"schur_matvec_variant", float(variant)))
        o = np.empty_like(v)
        _lib.check(m._lib.smc_schur_matvec(m._h, eta.ctypes.data_as(ctypes.c_void_p),
                                           v.ctypes.data_as(ctypes.c_void_p),
                                           o.ctypes.data_as(ctypes.c_void_p), 0))
        outs.append(o)
    assert _rel(outs[1], outs[0]) < 1e-11
    assert _rel(outs[2], outs[0]) < 1e-4
