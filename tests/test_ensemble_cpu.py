"""The multi-GPU path of the ensemble (one process per GPU, shards of the run
list, one gather on rank 0 at the end), run as two gloo ranks on the CPU with
a stand-in for the per-GPU march.  The single runs do not shard (replicas
only); their march is covered by the GPU tests."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _fake_march(sub, nsteps, **kw):
    """march_ensemble's result shape for each run, without a GPU."""
    return [dict(steps=nsteps, Nx=r["cfg"].Nx, amp=r["amp"], state=np.zeros(3),
                 device=kw.get("device")) for r in sub]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from specmc_gb300 import ensemble
        runs = ensemble.ensemble_configs(11, seed=3)
        out = ensemble.march_ensemble_sharded(runs, nsteps=7, march=_fake_march, device=rank)
        if rank == 0:
            q.put([(o["Nx"], o["amp"], o["rank"], o["steps"], o["device"], "state" in o) for o in out])
        else:
            q.put(out)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_is_a_round_robin_partition():
    from specmc_gb300.ensemble import shard
    parts = [shard(11, r, 3) for r in range(3)]
    assert sorted(i for p in parts for i in p) == list(range(11))
    assert parts[1] == [1, 4, 7, 10]
    with pytest.raises(ValueError):
        shard(11, 3, 3)


def test_sharded_ensemble_gathers_every_run_on_rank0():
    import torch.multiprocessing as mp
    from specmc_gb300 import ensemble
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res = next(g for g in got if g is not None)
    assert sum(g is None for g in got) == 1          # only rank 0 holds the gathered list
    runs = ensemble.ensemble_configs(11, seed=3)
    assert [(x[0], x[1]) for x in res] == [(r["cfg"].Nx, r["amp"]) for r in runs]
    assert [x[2] for x in res] == [i % 2 for i in range(11)]          # round robin over the ranks
    assert all(x[3] == 7 for x in res) and [x[4] for x in res] == [i % 2 for i in range(11)]
    assert not any(x[5] for x in res)                                  # states stay on their ranks


def _bench_worker(rank, world, port, q):
    import sys
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
        import bench
        q.put((rank, bench.max_over_ranks(1.5 + rank)))
    finally:
        dist.destroy_process_group()


def test_bench_times_the_slowest_replica():
    """bench.py under torchrun: each rank times its own replica and the line
    reports the slowest rank's time (world size 2, gloo)."""
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_bench_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 2.5, 1: 2.5}


def test_run_cost_orders_the_hard_runs_first():
    """The native driver starts the runs in decreasing estimated cost: the
    eta_T runs at high viscosity contrast and Rayleigh number before the
    isoviscous ones of the same grid, larger grids before smaller."""
    from specmc_gb300.config import ConvectionConfig
    from specmc_gb300.ensemble import ensemble_configs, run_cost
    c = lambda **kw: ConvectionConfig(**kw)
    assert run_cost(c(viscosity_model="eta_T", deta_T=1e4, Ra=1e6, Nx=64, Nz=48)) > \
        run_cost(c(viscosity_model="eta_T", deta_T=10.0, Ra=1e4, Nx=64, Nz=48)) > \
        run_cost(c(viscosity_model="eta_z", Nx=64, Nz=48)) > run_cost(c(viscosity_model="const", Nx=64, Nz=48))
    assert run_cost(c(viscosity_model="const", Nx=128, Nz=96)) > run_cost(c(viscosity_model="const", Nx=32, Nz=24))
    runs = ensemble_configs(256, seed=0)
    costs = sorted((run_cost(r["cfg"]) for r in runs), reverse=True)
    assert len(costs) == 256 and costs[0] > 100 * costs[-1]


def test_tuned_table_covers_the_ensemble_grids(tmp_path):
    """The autotuner's committed table gives every grid class of the seeded
    ensemble a CTA count among that grid's candidates; a missing table (or
    grid) gives None, so the driver falls back to its default."""
    from specmc_gb300 import ensemble, tune
    table = tune.load()
    for Nx, Nz in ensemble.GRIDS:
        c = tune.batch_ctas_for(Nx, Nz, table)
        assert c in tune.candidates(Nx), (Nx, Nz, c)
    assert tune.candidates(64) == sorted(set(tune.candidates(64)))
    assert all(16 <= c <= 304 for c in tune.candidates(128))
    assert tune.load(str(tmp_path / "none.json")) == {}
    assert tune.batch_ctas_for(64, 96, {}) is None
