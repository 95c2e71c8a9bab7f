"""The headline configurations at their own lengths, on the GPU.

* Configuration 2 (eta_T, deta_T = 1e3, Ra 1e4, 64x96, seeded conductive
  perturbation amp 3e-2, m = n = 1): the 200-step adaptive march against the
  reference's own 200-step record (tests/golden/long_etaT_64x96.npz: every
  dt, the diagnostics and the state every 20 steps, the counters), in both
  the plain FP64 form and the mixed form.
* Configuration 3 (internally heated 2:1 box, Lx = 4, Ra 1.25e4, H 1.5,
  eta_T deta_T 1e3, 64x96, seeded noise 1e-2 in m, n <= 8): the reference's
  first 60 steps (tests/golden/long_heated_2to1_64x96.npz, a record every
  10 steps) in both forms.

Bars: the reported quantities (Nu_top, Nu_energy, Vrms) to 1e-6 relative at
every recorded step -- the bar of this path -- in both forms; the plain form
follows the reference's algorithm step for step, so its dt, state and
control counters are held much tighter.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

KEYS = ("Nu_top", "Nu_bot", "Nu_energy", "urms", "umax", "amp")


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _cfg_kw(g):
    return {k[4:]: g[k].item() for k in g.files if k.startswith("cfg_")}


@pytest.fixture(scope="module")
def gb():
    from specmc_gb300 import _lib
    _lib.build()
    import specmc_gb300.api as api
    from specmc_gb300.config import ConvectionConfig
    return api, ConvectionConfig


def _march_against(gb, name, form, dt_tol, state_tol, diag_tol):
    api, CC = gb
    g = _load(name)
    m = api.build_model(CC(**_cfg_kw(g)), form=form)
    s = np.array(g["that0"], copy=True)
    ti = 0
    worst = dict(dt=0.0, state=0.0, diag=0.0)
    steps = list(g["trace_steps"])
    for n in range(len(g["dts"])):
        dt = api.production_dt(m, s)
        worst["dt"] = max(worst["dt"], abs(dt - g["dts"][n]) / g["dts"][n])
        s = m.step(s, dt)
        if n + 1 == steps[ti]:
            d = m.diagnostics(s)
            for c, key in enumerate(str(k) for k in g["trace_keys"]):
                if key in ("Nu_top", "Nu_energy", "urms"):
                    ref = g["trace"][ti, c]
                    worst["diag"] = max(worst["diag"], abs(d[key] - ref) / abs(ref))
            worst["state"] = max(worst["state"], _rel(s, g["trace_states"][ti]))
            ti += 1
    assert ti == len(steps)
    print("%s %s: worst rel dt %.2e, state %.2e, Nu/Vrms %.2e"
          % (name, form, worst["dt"], worst["state"], worst["diag"]))
    assert worst["dt"] <= dt_tol, worst
    assert worst["state"] <= state_tol, worst
    assert worst["diag"] <= diag_tol, worst
    c = m.counters()
    m.close()
    return g, c


def test_config2_200_steps_plain_matches_reference(gb):
    g, c = _march_against(gb, "long_etaT_64x96.npz", "plain", 1e-8, 1e-7, 1e-8)
    for key in ("n_refresh", "n_defect", "n_defect_failed", "n_defect_double_fail", "n_steps"):
        assert c[key] == int(g["ctr_" + key]), (key, c[key], int(g["ctr_" + key]))
    assert c["n_theta_nonconv"] == int(g["ctr_theta_n_nonconv"])


def test_config2_200_steps_mixed_matches_reference(gb):
    _march_against(gb, "long_etaT_64x96.npz", "mixed", 1e-6, 1e-5, 1e-6)


def test_config3_first_60_steps_plain_matches_reference(gb):
    g, c = _march_against(gb, "long_heated_2to1_64x96.npz", "plain", 1e-8, 1e-7, 1e-8)
    for key in ("n_refresh", "n_defect", "n_defect_failed", "n_steps"):
        assert c[key] == int(g["ctr_" + key]), (key, c[key], int(g["ctr_" + key]))


def test_config3_first_60_steps_mixed_matches_reference(gb):
    _march_against(gb, "long_heated_2to1_64x96.npz", "mixed", 1e-6, 1e-5, 1e-6)
