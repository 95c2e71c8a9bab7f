"""The batched engine: the refinement solves of many independent runs in one
cooperative launch (smc_march_many with the device's batcher), against the
same runs marched one engine launch per solve, and against the FP64 plain
form."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.fixture(scope="module")
def ens():
    from specmc_gb300 import _lib, ensemble
    _lib.build()
    runs = ensemble.ensemble_configs(256, seed=0)
    # two runs of every grid, mixed viscosity models, mostly coupled (eta_T):
    # they exercise both operators of the engine at four sizes
    pick, count = [], {}
    for i, r in enumerate(runs):
        c = r["cfg"]
        key = c.Nx
        if c.viscosity_model != "const" and count.get(key, 0) < 2:
            count[key] = count.get(key, 0) + 1
            pick.append(i)
    return ensemble, [runs[i] for i in pick]


def test_batched_equals_one_launch_per_solve(ens):
    """With the same CTAs per solve, a solve inside a batch (its own CTA range
    and group barrier) computes exactly what its own cooperative launch
    computes: the batched march equals the unbatched one bit for bit."""
    ensemble, runs = ens
    kw = dict(nsteps=6, form="mixed", concurrency=len(runs), batch_ctas=48)
    a = ensemble.march_ensemble_native(runs, batched=True, **kw)
    timing = a[0]["_timing"]
    assert timing["batch_solves"] > 0
    # batches held more than one solve on average
    assert timing["batch_solves"] > timing["batch_launches"]
    b = ensemble.march_ensemble_native(runs, batched=False, overrides=None, **kw)
    for x, y, run in zip(a, b, runs):
        # "amplitude" flags physical growth past 5x the seed (the run marches on)
        assert x["status"] == y["status"] and x["status"] in ("ok", "amplitude"), \
            (x["status"], y["status"])
        assert x["steps"] == y["steps"] == 6
        assert np.array_equal(x["state"], y["state"]), run["cfg"]


def test_batched_mixed_matches_plain(ens):
    """Each batched run agrees with the FP64 plain form to 1e-6 in Nu_top and
    Vrms after 6 steps (the two forms solve the same system to the same FP64
    tolerances)."""
    ensemble, runs = ens
    m = ensemble.march_ensemble_native(runs, nsteps=6, form="mixed", concurrency=len(runs))
    p = ensemble.march_ensemble_native(runs, nsteps=6, form="plain", concurrency=len(runs),
                                       batched=False)
    for x, y, run in zip(m, p, runs):
        assert x["status"] in ("ok", "amplitude") and y["status"] == x["status"]
        for key in ("Nu_top", "urms"):
            assert _rel(x["diag"][key], y["diag"][key]) <= 1e-6, (run["cfg"], key)
