"""specmc_gb300.heating / specmc_gb300.dissipation (the drop-in names of
physics/heating.py and physics/dissipation.py) against values the reference
computed (tests/golden/physics_helpers.json).  The model-dependent helpers
run on the oracle's model of the energy fixture's configuration."""
import json
import os

import numpy as np
import pytest

from oracle import specmc_oracle as O

from conftest import GOLDEN


@pytest.fixture(scope="module")
def ref():
    with open(os.path.join(GOLDEN, "physics_helpers.json")) as f:
        return json.load(f)


def _close(a, b, tol=1e-14):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return np.all(np.abs(a - b) <= tol * np.maximum(1.0, np.abs(b)))


def test_heating_closed_forms(ref):
    from specmc_gb300 import dissipation as DISS, heating as HEAT
    z = np.linspace(0.0, 1.0, 7)
    for H in (0.0, 1.5, 2.0, 4.0, -1.0):
        r = ref["H=%g" % H]
        assert _close(HEAT.conductive_theta(z, H), r["conductive_theta"])
        assert _close(HEAT.conductive_T(z, H), r["conductive_T"])
        assert _close(HEAT.mean_T_conductive(H), r["mean_T"])
        assert _close([HEAT.nu_bot_conductive(H), HEAT.nu_top_conductive(H)], [r["nu_bot"], r["nu_top"]])
        assert _close(HEAT.T_max_conductive(H), r["T_max"])
        assert _close([HEAT.nu_energy_steady(0.3, H), HEAT.nu_bot_energy_steady(0.3, H)],
                      [r["nu_energy"], r["nu_bot_energy"]])
        assert _close([DISS.nu_top_steady(0.3, H, 0.05), DISS.nu_bot_steady(0.3, H, 0.05)],
                      [r["nu_top_steady"], r["nu_bot_steady"]])
        assert HEAT.source_integral(H) == r["source_integral"]
        assert HEAT.source_coeffs(3, 4, H)[0, 0].real == r["source_00"]
        b = np.arange(12, dtype=complex)
        assert (HEAT.add_constant_source(b, 3, 4, H) is b) == (H == 0.0)


def test_dissipation_helpers(ref):
    from specmc_gb300 import dissipation as DISS
    from specmc_gb300.config import ConvectionConfig
    assert _close([DISS.single_mode_theta_integral(1e4, np.pi, np.pi, 1.0),
                   DISS.single_mode_theta_integral(3e5, 2 * np.pi, np.pi, 0.2),
                   DISS.single_mode_psi_integral(np.pi, 2 * np.pi, -3.0)], ref["single_mode"])
    rng = np.random.default_rng(2)
    prof = rng.uniform(0.5, 2.0, 5)
    cases = [None, np.ones((4, 5)), prof, np.tile(prof, (4, 1)), rng.uniform(0.5, 2.0, (4, 5))]
    assert [DISS.eta_class(c) for c in cases] == ref["eta_class"]
    got = [DISS.j9_2_bound(c, t, p) for c in ("const", "eta_z", "eta_xz", "other")
           for t, p in ((0.0, 0.0), (1e-8, 0.0), (0.0, 1e-3))]
    assert _close(got, ref["j9_2_bound"])
    g = np.load(os.path.join(GOLDEN, "energy_32x24.npz"))
    cfg = ConvectionConfig(Ra=1e4, Nx=32, Nz=24, viscosity_model="arrhenius", deta_T=1e3,
                           arrhenius_Ts=1.0, eta_min=1e-3, eta_max=1.0, dissipation_number=0.5,
                           internal_heating=1.0)
    m = O.build(cfg)
    assert _close(DISS.phi_z_tail(m, g["psi"], g["eta"]), ref["phi_z_tail"], 1e-10)
    sc = DISS.source_coeffs(m, g["psi"], g["eta"], Di=0.5)
    assert _close(np.linalg.norm(sc), ref["source_coeffs_norm"], 1e-11)
    assert _close(DISS.source_integral(m, sc), ref["source_coeffs_integral"], 1e-11)
    b = np.zeros(m.Nk * m.Nz, dtype=complex)
    out = DISS.add_dissipation_source(b, sc, 0.5).reshape(m.Nk, m.Nz)
    assert np.array_equal(out[:, :-2], sc[:, :-2]) and not out[:, -2:].any()
    assert DISS.add_dissipation_source(b, sc, 0.0) is b


def test_cfl_policy(ref):
    from specmc_gb300 import cfl_policy as CFL
    m = O.ConstModel(Ra=1e4, Nx=32, Nz=24)
    th = m.seed(amp=3e-2, m=1, n=1)
    got = [CFL.cfl_dt(m, th, safety=sf, dtmax=dm, clamp=cl)
           for sf in (0.4, 40.0, 500.0, -1.0) for dm in (4e-5, 1.0) for cl in (True, False)
           if not (sf < 0 and not cl)]
    assert _close(got, ref["cfl"], 1e-12)
    assert [CFL.clamp_safety(v) for v in (-3.0, 0.5, 40.0, 100.0)] == ref["clamp_safety"]
    assert (CFL.CFL_SAFETY_DEFAULT, CFL.CFL_SAFETY_MAX) == (40.0, 80.0)
