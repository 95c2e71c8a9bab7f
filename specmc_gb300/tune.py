"""Autotuner of the batched Krylov engine's launch shape.

A solve inside a batched launch (``engine_batch``) runs on its own range of
CTAs; how many is a trade: more CTAs per Fourier row shorten each Arnoldi
phase, fewer let more runs' solves share the GPU at once.  The best count
depends on the grid (Nk Fourier rows, Nz Chebyshev columns), so it is
measured: for each grid class, a small ensemble of same-size runs is marched
batched at each candidate count, and the count with the most aggregate
steps/s wins.  The table is kept in ``tuned.json`` beside this module (keys
"Nx x Nz"), read by the ensemble driver when no count is given, and
rewritten by ``python -m specmc_gb300.tune``.
"""
from __future__ import annotations

import json
import os
import time

HERE = os.path.dirname(os.path.abspath(__file__))
TUNE_PATH = os.path.join(HERE, "tuned.json")


def candidates(Nx, sms=152):
    """CTA counts tried for a grid of Nx columns: 1/2, 1, 2 and 3 CTAs per
    Fourier row (Nk = Nx/2 + 1), within [16, 2 * sms]."""
    nk = Nx // 2 + 1
    return sorted({max(16, min(2 * sms, int(r * nk))) for r in (0.5, 1, 2, 3)})


def load(path=TUNE_PATH):
    """-> the tuned table {"NxxNz": {"batch_ctas": c, ...}} ({} without one)."""
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f)


def batch_ctas_for(Nx, Nz, table=None):
    """-> the tuned CTAs per batched solve for an Nx x Nz grid, or None."""
    table = load() if table is None else table
    e = table.get("%dx%d" % (Nx, Nz))
    return int(e["batch_ctas"]) if e else None


def tune(grids=((32, 24), (64, 48), (64, 96), (128, 96)), nruns=16, nsteps=6, seed=0,
         device=0, path=TUNE_PATH, verbose=True):
    """Measure every candidate count on each grid class and write the table.

    Each class: ``nruns`` eta_T runs of that grid (Ra log-uniform in
    [1e4, 1e6], deta_T in [1, 1e4], seeded as the ensemble workload),
    marched ``nsteps`` steps batched in one native call per candidate (a
    short warm-up march first).  -> the table."""
    import numpy as np

    from . import ensemble
    from .config import ConvectionConfig
    rng = np.random.default_rng(seed)
    table = load(path)
    sms = ensemble.device_sms(device)
    for Nx, Nz in grids:
        runs = []
        for _ in range(nruns):
            cfg = ConvectionConfig(viscosity_model="eta_T", Nx=Nx, Nz=Nz,
                                   Ra=float(10.0 ** rng.uniform(4.0, 6.0)),
                                   deta_T=float(10.0 ** rng.uniform(0.0, 4.0)))
            runs.append(dict(cfg=cfg, amp=float(rng.uniform(1e-2, 5e-2)),
                             m=int(rng.integers(1, 5)), n=int(rng.integers(1, 5))))
        rates = {}
        for c in candidates(Nx, sms):
            ensemble.march_ensemble_native(runs[:2], nsteps=2, concurrency=2, batch_ctas=c,
                                           device=device, keep_states=False)
            t0 = time.perf_counter()
            res = ensemble.march_ensemble_native(runs, nsteps=nsteps, concurrency=nruns,
                                                 batch_ctas=c, device=device, keep_states=False)
            wall = res[0]["_timing"]["wall_s"] if res else time.perf_counter() - t0
            rates[c] = sum(r["steps"] for r in res) / wall
            if verbose:
                print("%dx%d  batch_ctas %3d  %8.1f steps/s" % (Nx, Nz, c, rates[c]), flush=True)
        best = max(rates, key=rates.get)
        table["%dx%d" % (Nx, Nz)] = dict(batch_ctas=int(best), steps_per_s=rates[best],
                                         tried={str(k): v for k, v in rates.items()},
                                         nruns=nruns, nsteps=nsteps)
    with open(path, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    return table


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--nruns", type=int, default=16)
    ap.add_argument("--nsteps", type=int, default=6)
    a = ap.parse_args()
    from . import _lib
    _lib.build()
    print(json.dumps(tune(nruns=a.nruns, nsteps=a.nsteps), indent=1))
