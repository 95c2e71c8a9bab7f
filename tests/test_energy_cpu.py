"""The energy-budget diagnostics (specmc_gb300.energy: physics/heating.py and
physics/dissipation.py of the reference) against values the reference wrote
(tests/golden/energy_32x24.npz), with the oracle model supplying the
transforms and Stokes solves.  The same functions run on the GPU model's
transforms in test_gpu_configs.py."""
import os

import numpy as np

from oracle import specmc_oracle as O
from specmc_gb300 import energy as EN
from specmc_gb300.config import ConvectionConfig

CFG = dict(Ra=1e4, Nx=32, Nz=24, viscosity_model="arrhenius", deta_T=1e3, arrhenius_Ts=1.0,
           eta_min=1e-3, eta_max=1.0, dissipation_number=0.5, internal_heating=1.0)


def _golden():
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "energy_32x24.npz"))


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def test_energy_diagnostics_match_reference():
    g = _golden()
    m = O.build(ConvectionConfig(**CFG))
    a0, b0, b1 = g["abc"]
    hb = EN.heating_balance(m, g["s3"], g["s2"], g["s1"], a0, b0, b1, H=1.0)
    for k, v in hb.items():
        assert abs(v - float(g["hb_" + k])) <= 1e-12 * max(1.0, abs(float(g["hb_" + k]))), k
    db = EN.dissipation_balance(m, g["s3"], g["s2"], g["s1"], a0, b0, b1, H=1.0, Di=0.5,
                                psi=g["psi"], eta=g["eta"])
    for k, v in db.items():
        assert abs(v - float(g["db_" + k])) <= 1e-11 * max(1.0, abs(float(g["db_" + k]))), k
    assert _rel(EN.phi_integral(m, g["psi"], g["eta"]), float(g["phi_int"])) < 1e-12
    assert _rel(EN.phi_integral(m, g["psi"]), float(g["phi_int_noeta"])) < 1e-12
    assert _rel(EN.pi_theta(m, g["psi"], g["s3"]), float(g["pi_theta"])) < 1e-12
    assert _rel(EN.pi_theta(m, g["psi"], g["s3"], dealias=False), float(g["pi_theta_plain"])) < 1e-12
    pc = EN.phi_coeffs(m, g["psi"], g["eta"])
    assert np.linalg.norm(pc - g["phi_coeffs"]) <= 1e-12 * np.linalg.norm(g["phi_coeffs"])
    # the flux profile solves Stokes itself (the oracle's solve: ~1e-9 of the reference's)
    z, q = EN.flux_profile(m, g["s3"], H=1.0)
    assert np.max(np.abs(q - g["q"])) <= 1e-7 * np.max(np.abs(g["q"]))
    nb, nt = EN.nu_pair(m, g["s3"])
    assert abs(nb - float(g["hb_nu_bot"])) < 1e-12 and abs(nt - float(g["hb_nu_top"])) < 1e-12
