"""specmc_gb300.viscosity / arrhenius / eta_bounds (the host versions of the
laws and the window the GPU eta kernels apply) against values the reference
computed on seeded points (tests/golden/rheology.npz)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(GOLDEN, "rheology.npz"))


def _rel(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_viscosity_laws(g):
    from specmc_gb300 import viscosity as VI
    assert _rel(VI.eta_exp_T(g["T"], 1e3), g["eta_exp_T"]) < 1e-15
    assert _rel(VI.eta_conductive_background(g["z"], 100.0), g["eta_background"]) < 1e-15
    assert np.array_equal(VI.eta_from_law("isoviscous", 100.0, g["z"]), g["eta_law_iso"])
    assert _rel(VI.eta_from_law("exp_T_depth", 100.0, g["z"]), g["eta_law_exp"]) < 1e-15
    with pytest.raises(NotImplementedError):
        VI.eta_from_law("arrhenius", 100.0, g["z"])


def test_arrhenius_laws(g):
    from specmc_gb300 import arrhenius as AR
    T, z = g["T"], g["z"]
    E, V, Ts = AR.arrhenius_E(1e3, 0.3), 0.7, 0.3
    got = [AR.arrhenius_E(1e3, 0.3), AR.arrhenius_C(1e3, 0.3), AR.cold_end_slope(1e3, 0.3),
           AR.slope_amplification(0.3), AR.infer_deta_T(5.0, 0.3), AR.infer_Ts(5.0, 1e3),
           AR.hot_end_contrast_V(T, z, E, V, Ts)]
    assert np.allclose(got, g["arr_scalars"], rtol=1e-14, atol=0.0)
    assert _rel(AR.arrhenius_exponent(T, 1e3, 0.3), g["arr_exponent"]) < 1e-15
    assert _rel(AR.eta_arrhenius_T(T, 1e3, 0.3), g["arr_eta"]) < 1e-15
    assert _rel(AR.arrhenius_exponent_V(T, z, E, V, Ts), g["arr_exponent_V"]) < 1e-15
    assert _rel(AR.eta_arrhenius_V(T, z, E, V, Ts), g["arr_eta_V"]) < 1e-15
    with pytest.raises(ValueError):
        AR.infer_Ts(5.0, 1.0)


def test_viscosity_window(g):
    from specmc_gb300 import arrhenius as AR
    from specmc_gb300 import eta_bounds as EB
    E, V, Ts = AR.arrhenius_E(1e3, 0.3), 0.7, 0.3
    w = [*EB.reachable_window(1e3), *EB.reachable_window_arrhenius(1e3, 1.0),
         *EB.reachable_window_arrhenius(1e3, 0.05), *EB.reachable_window_pv(E, V, Ts),
         *EB.effective_bounds(1e-3, 1e3)]
    assert np.allclose(w, g["windows"], rtol=1e-14, atol=0.0)
    eta = g["eta"]
    assert EB.n_clipped(eta, 1e-3, 1e3) == int(g["n_clipped"])
    out, n = EB.clip_eta(eta, 1e-3, 1e3)
    assert np.array_equal(out, g["clip"]) and n == int(g["clip_n"])
    inside = np.array([0.5, 2.0])
    assert EB.clip_eta(inside, 1e-3, 1e3)[0] is inside
    assert _rel(EB.smoothstep5(np.linspace(-0.5, 1.5, 21)), g["smoothstep"]) < 1e-15
    assert EB.n_in_transition(eta, 1e-3, 1e3, 1.5) == int(g["n_band"])
    out, n = EB.smooth_clip_eta(eta, 1e-3, 1e3, 1.5)
    assert _rel(out, g["smooth"]) < 1e-14 and n == int(g["smooth_n"])
