"""The CPU oracle against fixtures written by the SpecMC reference itself.

These pin the oracle (what the GPU path is tested against): if it drifts from the
reference, every GPU parity test downstream would be measuring against the
wrong thing.
"""
import os

import numpy as np
import pytest

from oracle import specmc_oracle as O

from conftest import GOLDEN


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


def test_basis_and_transforms():
    g = _load("transforms_16x12.npz")
    m = O.ConstModel(Ra=1e4, Nx=16, Nz=12)
    assert np.array_equal(m.D, g["D"])
    # cos of the host libm (CGL nodes): within an ulp of the fixture's machine
    np.testing.assert_allclose(m.V, g["V"], rtol=0.0, atol=1e-15)
    assert _rel(m.Vi, g["Vi"]) < 1e-15
    assert _rel(m.wq, g["wq"]) < 1e-14
    assert _rel(m.grid(g["cf"]), g["grid"]) < 1e-14
    assert _rel(m.coeffs(g["g"]), g["coeffs"]) < 1e-14
    assert _rel(m.synth_pad(g["cf"]), g["synth_pad"]) < 1e-14
    assert _rel(m.trunc_pad(g["gp"]), g["trunc_pad"]) < 1e-14
    psi, om = m.stokes(g["cf"])
    assert _rel(psi, g["psi"]) < 1e-13 and _rel(om, g["om"]) < 1e-13
    ux, uz = m.velocity(psi)
    assert _rel(ux, g["ux"]) < 1e-13 and _rel(uz, g["uz"]) < 1e-13
    assert _rel(m.step(g["cf"], 1e-4), g["step"]) < 1e-13
    assert _rel(m.seed(amp=3e-2, m=1, n=1), g["seed"]) < 1e-15


def test_coupled_operator():
    g = _load("coupled_ops_16x12.npz")
    m = O.CoupledModel(Nx=16, Nz=12, deta_T=1000.0)
    eta = m.eta_of(g["that"])
    assert _rel(eta, g["eta"]) < 1e-14
    assert _rel(np.array(m.G), g["G"]) < 1e-14
    Ms = m.eta_mats(eta)
    assert _rel(m.coeffs(eta), g["eta_c"]) < 1e-14
    assert _rel(m.schur_matvec(Ms, g["v"]), g["Av"]) < 1e-13
    assert _rel(m.assemble_schur(Ms), g["A"]) < 1e-13
    assert _rel(m.rhs_schur(g["that"]), g["b"]) < 1e-15
    lus = m.bfbt_lus(eta)
    N = m.Nz
    v = g["v"].copy()
    Pv = np.concatenate([__import__("scipy.linalg").linalg.lu_solve(
        lus[i], np.where(np.arange(N) < N - 2, v[i * N:(i + 1) * N], 0.0)) for i in range(m.Nk)])
    assert _rel(Pv, g["Pv"]) < 1e-12
    m2 = O.CoupledModel(Nx=16, Nz=12, deta_T=1000.0)
    psi, om = m2.stokes(g["that"])
    assert _rel(psi, g["psi"]) < 1e-9 and _rel(om, g["om"]) < 1e-9


def test_tala_operators():
    """The TALA route (compressibility='tala', Di = 0.7) operator by operator:
    reference state, L^(rho) Green functions, the distributed-form Schur
    matrix and its matrix-free action, the rho_bar^2 right-hand side, the
    unpacking, and the rho_bar-weighted temperature operator, preconditioner
    and adiabatic source after one step."""
    from specmc_gb300.config import ConvectionConfig
    g = _load("tala_ops_16x12.npz")
    cfg = ConvectionConfig(Ra=1e4, Nx=16, Nz=12, viscosity_model="eta_T", compressibility="tala",
                           dissipation_number=0.7, precond="legacy")
    m = O.build(cfg)
    assert m.tala and m.tala_a == g["tala_a"].item()
    np.testing.assert_allclose(m.rho_grid, g["rho_grid"], rtol=4.5e-16, atol=0.0)
    assert _rel(m.rho_c, g["rho_c"]) < 1e-15 and _rel(m.rho2_c, g["rho2_c"]) < 1e-15
    eta = m.eta_of(g["that"])
    assert _rel(eta, g["eta"]) < 1e-14
    assert _rel(np.array(m.Gt), g["G"]) < 1e-14
    Ms = m.eta_mats(eta)
    assert _rel(m.assemble_schur(Ms), g["A"]) < 1e-13
    assert _rel(m.schur_matvec(Ms, g["v"]), g["Av"]) < 1e-13
    assert _rel(m.rhs_schur(g["that"]), g["b"]) < 1e-15
    psi, om = m.unpack(g["v"])
    assert _rel(psi, g["psi_v"]) < 1e-14 and _rel(om, g["om_v"]) < 1e-15
    # one step: the Stokes defect correction (1e-8) and the temperature
    # FGMRES (1e-10) stop at tolerances, so the state agrees to their size
    th1 = m.step(g["that"], g["dt"].item())
    assert _rel(th1, g["that1"]) < 1e-9
    # the frozen velocity of that step is the same to the last bit (the
    # Stokes solve of the first step is direct from a fresh factorisation)
    assert _rel(m.theta_matvec(g["tv"]), g["theta_Av"]) < 1e-13
    assert _rel(m.theta_precond(g["tv"]), g["theta_Pv"]) < 1e-13
    assert _rel(m.tala_adiabatic(m.project_mirror(g["that"])), g["adiabatic"]) < 1e-13


def test_tala_reduces_to_boussinesq_at_zero_Di():
    """At Di = 0 the TALA operators are the Boussinesq ones (the limit the
    reference's own TALA self-test checks, stokes_tala.py:523-548)."""
    from specmc_gb300.config import ConvectionConfig
    g = _load("coupled_ops_16x12.npz")
    mb = O.CoupledModel(Nx=16, Nz=12, deta_T=1000.0)
    mt = O.CoupledModel(Nx=16, Nz=12, deta_T=1000.0, compressibility="tala")
    eta = mb.eta_of(g["that"])
    Mb, Mt = mb.eta_mats(eta), mt.eta_mats(eta)
    assert _rel(mt.assemble_schur(Mt), mb.assemble_schur(Mb)) < 1e-12
    assert _rel(mt.schur_matvec(Mt, g["v"]), mb.schur_matvec(Mb, g["v"])) < 1e-12
    assert np.array_equal(mt.rhs_schur(g["that"]), mb.rhs_schur(g["that"]))


CASES = ["const_32x24", "etaz_32x24", "etaT_32x24", "etaT_bfbt_32x24",
         "heated_2to1_32x24", "arrhenius_32x24", "smooth_32x24", "arrhenius_pv_32x24",
         "tala_const_32x24", "tala_etaz_32x24", "tala_etaT_32x24", "tala_arrhenius_32x24"]
DIAG_TOL = {}


def _cfg_from(g):
    kw = {k[4:]: g[k].item() for k in g.files if k.startswith("cfg_")}
    from specmc_gb300.config import ConvectionConfig
    return ConvectionConfig(**kw)


@pytest.mark.parametrize("case", CASES)
def test_march_matches_reference(case):
    g = _load("march_%s.npz" % case)
    cfg = _cfg_from(g)
    m = O.build(cfg)
    s = np.array(g["that0"], copy=True)
    worst = 0.0
    for n in range(len(g["dts"])):
        dt = O.production_dt(m, s)
        assert abs(dt - g["dts"][n]) <= 1e-9 * g["dts"][n], (n, dt, g["dts"][n])
        s = m.step(s, dt)
        worst = max(worst, _rel(s, g["states"][n]))
    d = m.diagnostics(s)
    assert worst < 1e-7, worst
    for key in ("Nu_top", "urms", "Nu_energy"):
        ref = g["diag_" + key].item()
        assert abs(d[key] - ref) <= DIAG_TOL.get(case, 1e-9) * abs(ref), (key, d[key], ref)
