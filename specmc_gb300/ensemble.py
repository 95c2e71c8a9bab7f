"""Ensembles of independent runs on one GPU (the batched workload).

Each run is its own model handle with its own CUDA stream.  The native
driver (``smc_march_many``, the default) marches all handles from a pool of
C++ threads; in the mixed form their Krylov refinement solves go to the
device's batcher, which runs the solves of many runs in one cooperative
launch, each run on its own CTAs with its own group barrier.  The Python
driver (``native=False``) drives the handles from Python threads instead,
each handle's engine capped at its share of the SMs.

The runs are independent -- nothing is exchanged between them while they
step -- so an ensemble shards across GPUs by partitioning the run list: one
process per GPU (torchrun) marches its shard (``march_ensemble_sharded``) and
the per-run results are gathered on rank 0 once, at the end.

``ensemble_configs`` draws the seeded mixed workload of 256 runs: grid from
{32x24, 64x48, 64x96, 128x96}, Ra log-uniform in [1e4, 1e6], deta_T
log-uniform in [1, 1e4], viscosity model uniform over const / eta_z / eta_T,
perturbation amplitude uniform in [1e-2, 5e-2] with modes m, n in 1..4.
"""
from __future__ import annotations

import ctypes
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import _lib, api
from . import _numerics as NUM
from .config import ConvectionConfig

__all__ = ["GRIDS", "MODELS", "ensemble_configs", "march_ensemble", "march_ensemble_native",
           "march_ensemble_sharded", "shard", "device_sms"]

GRIDS = ((32, 24), (64, 48), (64, 96), (128, 96))
MODELS = ("const", "eta_z", "eta_T")


def ensemble_configs(nruns=256, seed=0):
    """The seeded list of runs: dicts with ``cfg`` (ConvectionConfig) and the
    perturbation ``amp``, ``m``, ``n`` (drawn in this order per run)."""
    rng = np.random.default_rng(seed)
    runs = []
    for _ in range(int(nruns)):
        Nx, Nz = GRIDS[int(rng.integers(len(GRIDS)))]
        Ra = float(10.0 ** rng.uniform(4.0, 6.0))
        deta = float(10.0 ** rng.uniform(0.0, 4.0))
        vm = MODELS[int(rng.integers(len(MODELS)))]
        amp = float(rng.uniform(1e-2, 5e-2))
        m = int(rng.integers(1, 5))
        n = int(rng.integers(1, 5))
        cfg = ConvectionConfig(viscosity_model=vm, Nx=Nx, Nz=Nz, Ra=Ra, deta_T=deta)
        runs.append(dict(cfg=cfg, amp=amp, m=m, n=n))
    return runs


def device_sms(device=0):
    """Streaming multiprocessors of ``device``."""
    import torch
    return int(torch.cuda.get_device_properties(device).multi_processor_count)


def _build(cfg, form, device, overrides):
    """api.build_model, with constructor keywords of the model replaced by
    ``overrides`` (e.g. tighter solver tolerances) when given."""
    if not overrides:
        return api.build_model(cfg, form=form, device=device)
    spec = api.model_spec(cfg)
    kw = dict(spec["kwargs"])
    kw.update(overrides)
    return api.MODEL_MODULES[spec["model"]].build(**kw, form=form, device=device)


def _march_one(run, nsteps, form, device, cap, safety, dtmax, chunk, max_wall, overrides=None):
    """One run: CFL-limited steps in chunks of ``chunk``; after each chunk the
    state is checked.  The run is flagged when max|theta| on the grid exceeds
    AMP_LIMIT x its initial value (the reference driver's abort threshold,
    specmc/_numerics.py:139-140; the ensemble keeps marching such a run and
    reports it), and it stops, flagged, when the state is non-finite, the
    march stalls, or it has used ``max_wall`` seconds."""
    t0 = time.perf_counter()
    model = _build(run["cfg"], form, device, overrides)
    try:
        lib, h = model._lib, model._h
        if cap > 0:
            _lib.check(lib.smc_set_option(h, b"engine_ctas", float(cap)))
        th = np.ascontiguousarray(model.seed(amp=run["amp"], m=run["m"], n=run["n"]))
        amp0 = float(np.abs(model.grid(th)).max())
        _lib.check(lib.smc_set_state(h, th.ctypes.data_as(ctypes.c_void_p), _lib.SMC_HOST))
        t1 = time.perf_counter()
        info = _lib.SmcMarchInfo()
        s = np.empty_like(th)
        steps, status = 0, "ok"
        while steps < nsteps:
            k = min(int(chunk), int(nsteps) - steps)
            _lib.check(lib.smc_advance(h, 1e300, k, float(safety), float(dtmax), ctypes.byref(info)))
            steps += int(info.steps)
            _lib.check(lib.smc_get_state(h, s.ctypes.data_as(ctypes.c_void_p), _lib.SMC_HOST))
            if not np.all(np.isfinite(s)) or not np.isfinite(info.t):
                status = "non-finite"
                break
            if status == "ok" and float(np.abs(model.grid(s)).max()) > NUM.AMP_LIMIT * max(amp0, 1e-300):
                status = "amplitude"
            if info.steps < k:
                status = "stalled"
                break
            if max_wall and time.perf_counter() - t1 > max_wall:
                status = "time"
                break
        t2 = time.perf_counter()
        finite = bool(np.all(np.isfinite(s)))
        diag = model.diagnostics(s) if finite else {}
        return dict(steps=steps, t=float(info.t), dt=float(info.dt), build_s=t1 - t0,
                    march_s=t2 - t1, state=s, diag=diag, finite=finite,
                    flagged=status != "ok", status=status, counters=model.counters())
    finally:
        model.close()


def run_cost(cfg):
    """A rough relative cost of marching ``cfg`` (for ordering only): grid
    size times a factor of the viscosity model, which for eta_T grows with the
    viscosity contrast and the Rayleigh number (the BFBT iteration counts and
    the dense rescues of the hard runs)."""
    cells = (cfg.Nx // 2 + 1) * cfg.Nz
    vm = cfg.viscosity_model
    if vm == "const":
        return cells
    if vm == "eta_z":
        return 4.0 * cells
    return 16.0 * cells * (1.0 + np.log10(max(cfg.deta_T, 1.0))) * np.sqrt(cfg.Ra / 1e4)


def march_ensemble_native(runs, nsteps=100, form="mixed", concurrency=16, safety=None,
                          dtmax=None, device=0, batched=True, check_every=5, overrides=None,
                          batch_ctas=None, keep_states=True, longest_first=True):
    """March every run of ``runs`` for ``nsteps`` CFL-limited steps in one
    native call (``smc_march_many``: ``concurrency`` C++ threads; with
    ``batched`` the mixed form's refinement solves of all runs go through the
    device's batcher).  Every run is checked every ``check_every`` steps: a
    non-finite state stops it ('non-finite'); max|theta| above AMP_LIMIT x its
    initial value flags it ('amplitude', the reference driver's abort
    threshold, specmc/_numerics.py:139-140) and it marches on.  No run is cut
    short for time.  With ``longest_first`` the worker threads take the runs in
    decreasing ``run_cost`` (a long run drawn last would stretch the wall time;
    every run's result is the same in any order).  Returns one result dict per
    run, in the order of ``runs`` (as march_ensemble), and, under the key
    ``"_timing"`` of the first, the march's wall time and the batcher's launch
    statistics."""
    safety = NUM.CFL_SAFETY if safety is None else float(safety)
    dtmax = NUM.DTMAX if dtmax is None else float(dtmax)
    lib = _lib.load()
    from . import tune
    table = tune.load() if batch_ctas is None else {}
    models, t_build = [], []
    try:
        for run in runs:
            t0 = time.perf_counter()
            model = _build(run["cfg"], form, device, overrides)
            models.append(model)
            if batch_ctas and model.form == "mixed":
                # CTAs per solve, batched or not
                _lib.check(lib.smc_set_option(model._h, b"engine_batch_ctas", float(batch_ctas)))
                _lib.check(lib.smc_set_option(model._h, b"engine_ctas", float(batch_ctas)))
            elif model.form == "mixed":
                c = tune.batch_ctas_for(run["cfg"].Nx, run["cfg"].Nz, table)
                if c:        # the autotuned count of this grid (specmc_gb300/tuned.json)
                    _lib.check(lib.smc_set_option(model._h, b"engine_batch_ctas", float(c)))
            th = np.ascontiguousarray(model.seed(amp=run["amp"], m=run["m"], n=run["n"]))
            _lib.check(lib.smc_set_state(model._h, th.ctypes.data_as(ctypes.c_void_p),
                                         _lib.SMC_HOST))
            t_build.append(time.perf_counter() - t0)
        order = list(range(len(models)))
        if longest_first:
            order.sort(key=lambda i: -run_cost(runs[i]["cfg"]))
        hs = (ctypes.c_void_p * len(models))(*[models[i]._h for i in order])
        res_ord = (_lib.SmcRunResult * len(models))()
        b0 = [ctypes.c_longlong() for _ in range(3)]
        _lib.check(lib.smc_batch_stats(int(device), *[ctypes.byref(x) for x in b0]))
        t0 = time.perf_counter()
        _lib.check(lib.smc_march_many(hs, len(models), int(nsteps), safety, dtmax,
                                      float(NUM.AMP_LIMIT), int(check_every), int(concurrency),
                                      1 if batched else 0, res_ord))
        wall = time.perf_counter() - t0
        b1 = [ctypes.c_longlong() for _ in range(3)]
        _lib.check(lib.smc_batch_stats(int(device), *[ctypes.byref(x) for x in b1]))
        res = [None] * len(models)
        for j, i in enumerate(order):
            res[i] = res_ord[j]
        out = []
        for i, (model, r) in enumerate(zip(models, res)):
            s = np.empty((model.Nk, model.Nz), dtype=np.complex128)
            _lib.check(lib.smc_get_state(model._h, s.ctypes.data_as(ctypes.c_void_p), _lib.SMC_HOST))
            finite = bool(np.all(np.isfinite(s)))
            status = _lib.RUN_STATUS[int(r.status)]
            out.append(dict(steps=int(r.steps), t=float(r.t), dt=float(r.dt), build_s=t_build[i],
                            march_s=float(r.seconds), state=s if keep_states else None,
                            diag=model.diagnostics(s) if finite else {}, finite=finite,
                            flagged=status != "ok", status=status, amp0=float(r.amp0),
                            amp=float(r.amp), counters=model.counters()))
        if out:
            out[0]["_timing"] = dict(wall_s=wall, batch_launches=b1[0].value - b0[0].value,
                                     batch_solves=b1[1].value - b0[1].value,
                                     batch_ctas=b1[2].value - b0[2].value)
        return out
    finally:
        for model in models:
            model.close()


def march_ensemble(runs, nsteps=100, form="mixed", concurrency=8, safety=None, dtmax=None,
                   device=0, engine_ctas=None, chunk=5, max_wall=None, on_done=None,
                   overrides=None):
    """March every run of ``runs`` for ``nsteps`` CFL-limited steps, up to
    ``concurrency`` at a time.  Returns one result dict per run (steps, t,
    build and march seconds, final state, diagnostics, status and flag,
    counters); flagged runs stop early and are kept in the list.

    ``engine_ctas`` caps each handle's Krylov engine; the default gives each
    concurrent run an equal share of two CTAs per SM.  ``on_done(i, result)``
    is called as each run finishes.  ``overrides``: model constructor keywords
    to replace for every run (e.g. ``stokes_rtol``, ``theta_rtol``)."""
    safety = NUM.CFL_SAFETY if safety is None else float(safety)
    dtmax = NUM.DTMAX if dtmax is None else float(dtmax)
    concurrency = max(1, int(concurrency))
    if engine_ctas is None:
        engine_ctas = max(1, (2 * device_sms(device)) // concurrency) if concurrency > 1 else 0
    out = [None] * len(runs)

    def work(i):
        out[i] = _march_one(runs[i], nsteps, form, device, int(engine_ctas), safety, dtmax,
                            chunk, max_wall, overrides)
        if on_done is not None:
            on_done(i, out[i])

    if concurrency == 1:
        for i in range(len(runs)):
            work(i)
    else:
        with ThreadPoolExecutor(max_workers=concurrency) as ex:
            for f in [ex.submit(work, i) for i in range(len(runs))]:
                f.result()
    return out


def shard(nruns, rank, world):
    """-> the run indices of ``rank`` out of ``world``: round robin (i = rank,
    rank + world, ...), which spreads the grid sizes and models of the seeded
    list evenly over the GPUs."""
    if not (0 <= int(rank) < int(world)):
        raise ValueError("rank %r outside world size %r" % (rank, world))
    return list(range(int(rank), int(nruns), int(world)))


def march_ensemble_sharded(runs, nsteps=100, rank=None, world=None, group=None,
                           keep_states=False, march=None, **kw):
    """One process per GPU: march this rank's shard of ``runs``
    (``march_ensemble(..., **kw)`` on this process's GPU, ``device`` in ``kw``)
    and gather the per-run results on rank 0 with one host-side gather after
    every run has finished; nothing is exchanged while the runs step.

    -> on rank 0 the results of all runs in run order (each with its
    ``rank``), elsewhere None.  The final states stay on their ranks unless
    ``keep_states``.  ``rank``/``world`` default to the initialised
    torch.distributed group (a single process without one); ``march``
    replaces march_ensemble (same call), e.g. to test the gather without a GPU."""
    dist = None
    if rank is None or world is None:
        import torch.distributed as dist
        if dist.is_available() and dist.is_initialized():
            rank = dist.get_rank(group) if rank is None else rank
            world = dist.get_world_size(group) if world is None else world
        else:
            rank, world, dist = 0, 1, None
    idx = shard(len(runs), rank, world)
    res = (march or march_ensemble)([runs[i] for i in idx], nsteps=nsteps, **kw)
    mine = []
    for i, r in zip(idx, res):
        r = dict(r, rank=int(rank))
        if not keep_states:
            r.pop("state", None)
        mine.append((i, r))
    if world == 1:
        parts = [mine]
    else:
        if dist is None:
            import torch.distributed as dist
        parts = [None] * world if rank == 0 else None
        dist.gather_object(mine, parts, dst=0, group=group)
    if rank != 0:
        return None
    out = [None] * len(runs)
    for part in parts:
        for i, r in part:
            out[i] = r
    return out


def _main(argv=None):
    """python -m specmc_gb300.ensemble [--runs 256] [--steps 100] ...: march the
    seeded ensemble and print one JSON summary line."""
    import argparse
    import collections
    import json
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--runs", type=int, default=256)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--form", default="mixed", choices=("mixed", "plain"))
    ap.add_argument("--concurrency", type=int, default=8)
    ap.add_argument("--engine-ctas", type=int, default=None)
    ap.add_argument("--max-wall", type=float, default=None,
                    help="seconds after which a run stops, flagged 'time' (Python driver)")
    ap.add_argument("--driver", default="native", choices=("native", "python"),
                    help="native: smc_march_many (C++ threads, batched engine); "
                         "python: Python threads, one engine launch per solve")
    ap.add_argument("--no-batch", action="store_true", help="native driver without the batcher")
    ap.add_argument("--given-order", action="store_true",
                    help="native driver: start the runs in list order (default: longest first)")
    a = ap.parse_args(argv)
    import os
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    runs = ensemble_configs(a.runs, a.seed)
    if world > 1:          # under torchrun: one shard per GPU, gathered on rank 0
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", init_method="env://", world_size=world, rank=rank)
    t0 = time.perf_counter()
    if a.driver == "native":
        res = march_ensemble_sharded(runs, nsteps=a.steps, rank=rank, world=world, form=a.form,
                                     concurrency=a.concurrency, device=local,
                                     batched=not a.no_batch, march=march_ensemble_native,
                                     longest_first=not a.given_order)
    else:
        res = march_ensemble_sharded(runs, nsteps=a.steps, rank=rank, world=world, form=a.form,
                                     concurrency=a.concurrency, engine_ctas=a.engine_ctas,
                                     max_wall=a.max_wall, device=local)
    wall = time.perf_counter() - t0
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([wall], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        wall = float(t.item())
        dist.destroy_process_group()
    if rank != 0:
        return
    steps = sum(r["steps"] for r in res)
    by = collections.defaultdict(list)
    for run, r in zip(runs, res):
        by["%dx%d %s" % (run["cfg"].Nx, run["cfg"].Nz, run["cfg"].viscosity_model)].append(
            1e3 * r["march_s"] / max(r["steps"], 1))
    timing = res[0].get("_timing") if res and res[0] else None
    print(json.dumps(dict(
        runs=len(runs), n_gpus=world, steps=steps, wall_s=wall, steps_per_s=steps / wall, form=a.form,
        driver=a.driver, batched=a.driver == "native" and not a.no_batch, march=timing,
        concurrency=a.concurrency, build_s=sum(r["build_s"] for r in res),
        status=dict(collections.Counter(r["status"] for r in res)),
        median_ms_per_step={k: float(np.median(v)) for k, v in sorted(by.items())})))


if __name__ == "__main__":
    _main()
