"""Model-level workflow calls of the GPU models: run, mirror_error,
dissipation_eta (the viscosity the last Stokes solve consumed) and
dissipation_phi, against the reference's records
(tests/golden/drivers_32x24.npz) and the oracle."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    from specmc_gb300 import _lib
    _lib.build()
    import specmc_gb300.api as api
    from specmc_gb300.config import ConvectionConfig
    return api, ConvectionConfig


def test_run_and_mirror_error_on_gpu(gb):
    api, CC = gb
    g = np.load(os.path.join(GOLDEN, "drivers_32x24.npz"))
    m = api.build_model(CC(viscosity_model="const", Nx=32, Nz=24))
    s, hist = m.run(g["that0"], tstop=30 * 4e-5 * 0.999, safety=0.5, dtmax=4e-5, cadence=10,
                    verbose=False)
    keys = [str(k) for k in g["keys"]]
    got = np.array([[h[k] for k in keys] for h in hist])
    assert got.shape == g["hist"].shape
    assert np.abs(got - g["hist"]).max() <= 1e-10 * np.abs(g["hist"]).max()
    assert m.mirror_error(s) < 1e-13
    assert abs(m.mirror_error(g["odd"]) - g["mirror_odd"].item()) <= 1e-13
    assert m.dissipation_eta() is None


def test_dissipation_eta_is_the_consumed_field(gb):
    from oracle import specmc_oracle as O
    api, CC = gb
    cz = CC(viscosity_model="eta_z", deta_T=100.0, Nx=32, Nz=24)
    ez = api.build_model(cz).dissipation_eta()
    assert ez.shape == (24,)
    assert np.abs(ez - O.build(cz).eta_grid).max() <= 1e-14 * np.abs(ez).max()
    ct = CC(viscosity_model="eta_T", Nx=32, Nz=24, dissipation_number=0.5)
    m, o = api.build_model(ct), O.build(ct)
    before = m.dissipation_eta()
    assert before.shape == (24,)
    assert np.abs(before - o.eta_grid).max() <= 1e-14 * np.abs(before).max()
    th = m.seed(amp=3e-2, m=1, n=1)
    m.stokes(th)
    assert m.theta.scheme == "bdf2" and m.theta.rtol == 1e-10 and m.theta.n_solves == 0
    after = m.dissipation_eta()
    assert after.shape == (32, 24)
    ref = o.eta_of(th)
    assert np.abs(after - ref).max() <= 1e-13 * np.abs(ref).max()
    psi, _ = o.stokes(th)
    phi = m.dissipation_phi(psi)
    phi_o = O.phi_padded(o, psi, ref)
    assert phi.shape == (64, 24)
    assert np.abs(phi - phi_o).max() <= 1e-10 * np.abs(phi_o).max()


def test_single_mode_analytic_solution_on_gpu(gb):
    """The single-mode known answers of core/rbc_galerkin.py:500-513 and
    physics/dissipation.py:495-517 on the GPU model: for theta = Theta
    cos(pi x) sin(pi z), psi = -Ra pi/g^2 Theta sin(pi x) sin(pi z),
    u_z = Ra pi^2/g^2 theta and <Phi> = Ra <theta u_z> = Ra^2 pi^2/(4 g^2) Theta^2,
    g = 2 pi^2."""
    from specmc_gb300 import energy
    api, CC = gb
    Ra, Theta, k = 1e4, 0.7, np.pi
    m = api.build_model(CC(viscosity_model="const", Ra=Ra, Nx=16, Nz=32))
    X, Z = np.meshgrid(m.x, m.z, indexing="ij")
    g = 2.0 * k * k
    th = Theta * np.cos(k * X) * np.sin(k * Z)
    that = m.coeffs(th)
    psi, _ = m.stokes(that)
    psi_ref = -Ra * k / g ** 2 * Theta * np.sin(k * X) * np.sin(k * Z)
    assert np.abs(m.grid(psi) - psi_ref).max() <= 1e-11 * np.abs(psi_ref).max()
    _, uz = m.velocity(psi)
    uz_ref = Ra * k * k / g ** 2 * th
    assert np.abs(uz - uz_ref).max() <= 1e-11 * np.abs(uz_ref).max()
    phi_ref = Ra ** 2 * k * k / (4.0 * g ** 2) * Theta ** 2
    assert abs(energy.phi_integral(m, psi) - phi_ref) <= 1e-10 * phi_ref
    assert abs(energy.pi_theta(m, psi, that) - phi_ref) <= 1e-10 * phi_ref


def test_forced_bfbt_rescue(gb):
    """Failure injection on the host, the reference's own check
    (models/coupled_model.py:955-969): with a one-iteration FGMRES budget the
    BFBT Stokes solve cannot converge, so the rescue must fire once and
    return the lagged-LU solution, equal to the legacy route's."""
    from oracle import specmc_oracle as O
    from specmc_gb300.solver import RBCCoupled
    api, CC = gb
    mr = RBCCoupled(Nx=16, Nz=12, deta_T=1000.0, precond="bfbt", stokes_maxiter=1)
    th = mr.seed(amp=1e-2, m=1, n=1)
    psi_r, _ = mr.stokes(th)
    c = mr.counters()
    assert c["n_bfbt_solves"] == 1 and c["n_bfbt_rescue"] == 1 and c["n_refresh"] == 1
    ml = RBCCoupled(Nx=16, Nz=12, deta_T=1000.0, precond="legacy")
    psi_l, _ = ml.stokes(th)
    assert np.abs(psi_r - psi_l).max() <= 1e-12 * np.abs(psi_l).max()
    psi_o, _ = O.CoupledModel(Nx=16, Nz=12, deta_T=1000.0, precond="legacy").stokes(th)
    assert np.abs(psi_r - psi_o).max() <= 1e-8 * np.abs(psi_o).max()



def test_mixed_rescue_then_lu_preconditioned(gb):
    """The mixed form with a one-iteration BFBT budget: its first Stokes solve
    fails (FP32, then FP64) and is rescued by the dense route (refresh +
    defect correction); the later solves are FP64 FGMRES solves preconditioned
    by that factor, refactored only when such a solve fails (then the legacy
    route for a while).  The march equals the plain legacy route's to the
    solver tolerances, and not every solve refactors."""
    from specmc_gb300.solver import RBCCoupled
    mm = RBCCoupled(Nx=32, Nz=24, deta_T=1000.0, stokes_maxiter=1, form="mixed")
    mp = RBCCoupled(Nx=32, Nz=24, deta_T=1000.0, precond="legacy")
    sm = mm.seed(amp=3e-2, m=1, n=1)
    sp = np.array(sm, copy=True)
    steps = 12
    for _ in range(steps):
        dt = mp.production_dt(sp)
        sp = mp.step(sp, dt)
        sm = mm.step(sm, dt)
    c = mm.counters()
    assert c["n_bfbt_rescue"] >= 1 and c["n_refresh"] < c["n_stokes"], c
    assert np.abs(sm - sp).max() <= 1e-7 * np.abs(sp).max()
    dm, dp = mm.diagnostics(sm), mp.diagnostics(sp)
    for key in ("Nu_top", "urms"):
        assert abs(dm[key] - dp[key]) <= 1e-7 * abs(dp[key]), (key, dm[key], dp[key])