#!/usr/bin/env python
"""Benchmark of the SpecMC time step on GB300: steps/s of the coupled eta(T)
workload (Ra = 1e4, deta_T = 1000, 1x1 box, Nx = 64 x Nz = 96, seeded
conductive perturbation amp = 3e-2 m = n = 1; the 200-step adaptive march).

One bench "step" is one CFL-limited time step of that march (production_dt +
step: eta(T), the coupled Stokes solve, the BDF2 temperature solve) in the
mixed form (BFBT-preconditioned FGMRES as FP32 iterative refinement of the
FP64 system, one persistent launch per solve).  W warm-up steps run first; the
K timed steps are the steps W+1 .. W+K of the march.

  value  steps/s with the state resident in HBM (device-resident march,
         CUDA events on the handle's stream around each step; an L2 flush
         runs between steps, outside the events).
  e2e    the same steps through the public API with host (pinned) buffers:
         dt = api.production_dt(model, s); s = model.step(s, dt) -- the
         state crosses host<->device every step.
  plain_fp64   the same march in the FP64 plain form (the reference's route:
               lagged dense LU + defect correction), timed as `value`.
  batched      a bounded sample of the many-run ensemble (the first 64 runs
               of the seeded 256-run list, 20 steps each) through the batched
               engine, against the plain form on the same sample.

``--impl reference`` times the CPU oracle (the restatement of the reference
NumPy/SciPy path, all host threads) on the same workload and prints the same
line with ``"impl": "reference"``.  Under torchrun (N > 1) the single run is
replicated per GPU (replicas only, no collective on the data path).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "steps/sec, mixed-precision vs FP64 GPU path at <=1e-6 rel Nu/Vrms error"
WORKLOAD = dict(viscosity_model="eta_T", deta_T=1000.0, Ra=1e4, Nx=64, Nz=96)
SEED = dict(amp=3e-2, m=1, n=1)
L2_BYTES = 129 * 1024 * 1024
# DRAM bytes (read + write) per launch of the dominant kernels: ncu
# dram__bytes_read.sum + dram__bytes_write.sum, mean over the captured
# launches of this workload (--clock-control none, a few launches of one
# kernel after the warm-up steps); TRAFFIC_SOURCE names the committed summary
DRAM_BYTES_PER_LAUNCH = {"engine_stokes": 28.28e6, "engine_theta": 3.46e6}
TRAFFIC_SOURCE = "profiles/kernels_64x96_small.md (Stokes), profiles/engine_64x96.md (theta)"


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured (MEASURED_PEAKS.json)"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms (a thread)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU side
def cpu_oracle_rate(steps, warmup, threads=None):
    """steps/s of the CPU oracle on the workload (steps W+1..W+K), in a fresh
    interpreter so that no CUDA context is inherited."""
    code = r"""
import json, os, sys, time
sys.path.insert(0, %r)
from oracle import specmc_oracle as O
from specmc_gb300.config import ConvectionConfig
cfg = ConvectionConfig(**%r)
m = O.build(cfg)
s = m.seed(**%r)
for _ in range(%d):
    s = m.step(s, O.production_dt(m, s))
t0 = time.perf_counter()
for _ in range(%d):
    s = m.step(s, O.production_dt(m, s))
el = time.perf_counter() - t0
print(json.dumps(dict(steps=%d, seconds=el)))
""" % (ROOT, WORKLOAD, SEED, warmup, steps, steps)
    env = dict(os.environ)
    if threads:
        for v in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS"):
            env[v] = str(threads)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError("CPU oracle failed:\n" + r.stderr[-2000:])
    d = json.loads(r.stdout.strip().splitlines()[-1])
    return d["steps"] / d["seconds"], d


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    cores = os.cpu_count()
    # the same march steps as the GPU arm: warm-up steps 1..W, timed W+1..W+K
    steps = args.steps if args.ref_steps is None else max(1, args.ref_steps)
    warm = args.warmup if args.ref_warmup is None else args.ref_warmup
    rate, d = cpu_oracle_rate(steps, warm, threads=cores)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "steps/s",
        "n_gpus": args.gpus, "steps": steps, "warmup": warm,
        "ms_per_step": 1e3 / rate, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded conductive perturbation)",
        "config": dict(workload="eta_T 64x96 Ra=1e4 deta_T=1e3, 200-step adaptive march",
                       sample="steps %d..%d" % (warm + 1, warm + steps), **WORKLOAD),
        "cpu_baseline": {"value": rate, "unit": "steps/s", "cores": cores, "kind": "port",
                         "sample": "oracle restatement (NumPy/SciPy, LAPACK on all host threads), "
                                   "steps %d..%d of the march" % (warm + 1, warm + steps)},
        "e2e": {"value": rate, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def max_over_ranks(x):
    """-> the maximum of ``x`` over the ranks of the initialised process group
    (``x`` without one): the timed region of N replicas is the slowest rank's.
    A CUDA tensor carries it over NCCL, a host tensor over gloo."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ GPU side
def run_ours(args, rank, world):
    import ctypes

    import numpy as np
    import torch

    from specmc_gb300 import _lib, api
    from specmc_gb300.config import ConvectionConfig

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    _lib.build()
    cfg = ConvectionConfig(**WORKLOAD)
    n_c = (cfg.Nx // 2 + 1) * cfg.Nz

    # CPU baseline first (rank 0, N = 1 only): a fresh interpreter
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        # the steps this arm times (at most 20 of them), after the same warm-up
        k = args.cpu_steps if args.cpu_steps else min(args.steps, 20)
        rate, d = cpu_oracle_rate(k, args.warmup, threads=os.cpu_count())
        cpu = {"value": rate, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "oracle restatement (NumPy/SciPy, LAPACK on all host threads), steps "
                         "%d..%d of the same march (%.1f s timed)"
                         % (args.warmup + 1, args.warmup + k, d["seconds"])}

    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    def timed_march(form, steps, warmup, profile):
        m = api.build_model(cfg, form=form, device=local)
        lib = m._lib
        th0 = m.seed(**SEED)
        stream = torch.cuda.ExternalStream(lib.smc_stream(m._h), device=local)
        th_d = torch.from_numpy(np.ascontiguousarray(th0)).to("cuda")
        _lib.check(lib.smc_set_state(m._h, ctypes.c_void_p(th_d.data_ptr()), _lib.SMC_DEVICE))
        info = _lib.SmcMarchInfo()
        for _ in range(warmup):
            _lib.check(lib.smc_advance(m._h, 1e30, 1, 40.0, 4e-5, ctypes.byref(info)))
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        c0 = m.counters()["n_kernel_launches"]
        if profile:
            # 2: only the engine's launches (two events per solve); 1: every region
            if args.phases and form == "mixed" and profile == 1:
                _lib.check(lib.smc_set_option(m._h, b"engine_phase_profile", 1.0))
            _lib.check(lib.smc_profile(m._h, profile))
        evs = []
        torch.cuda.synchronize()
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
            _lib.check(lib.smc_advance(m._h, 1e30, 1, 40.0, 4e-5, ctypes.byref(info)))
            with torch.cuda.stream(stream):
                b.record(stream)
            evs.append((a, b))
        torch.cuda.synchronize()
        step_ms = sorted(a.elapsed_time(b) for a, b in evs)
        ms_total = sum(step_ms)
        launches = m.counters()["n_kernel_launches"] - c0
        prof = []
        if profile:
            name, ms, nl = ctypes.c_char_p(), ctypes.c_double(), ctypes.c_longlong()
            work, isb = ctypes.c_double(), ctypes.c_int()
            for slot in range(64):
                _lib.check(lib.smc_profile_get(m._h, slot, ctypes.byref(name), ctypes.byref(ms),
                                               ctypes.byref(nl), ctypes.byref(work), ctypes.byref(isb)))
                if not name.value:
                    break
                prof.append(dict(name=name.value.decode(), ms=ms.value, launches=nl.value,
                                 work=work.value, is_bytes=isb.value))
            _lib.check(lib.smc_profile(m._h, 0))
        state = torch.empty((m.Nk, m.Nz), dtype=torch.complex128, device="cuda")
        _lib.check(lib.smc_get_state(m._h, ctypes.c_void_p(state.data_ptr()), _lib.SMC_DEVICE))
        diag = m.diagnostics(state.cpu().numpy())
        ms_total = max_over_ranks(ms_total)
        return dict(ms=ms_total, launches=launches, prof=prof, diag=diag, m=m, th0=th0,
                    step_ms=step_ms)

    clocks = ClockSampler(local)
    clocks.start()
    # the timed march: CUDA events around the engine launches only
    M = timed_march("mixed", args.steps, args.warmup, 2)
    clk = clocks.stop()
    # the same steps again with every kernel region timed (the per-region
    # table; its events would perturb the timed march)
    R = timed_march("mixed", args.steps, args.warmup, 1)
    P = timed_march("plain", args.steps, args.warmup, 0) if not args.no_plain else None
    value = world * args.steps / (M["ms"] / 1e3)

    # e2e through the public API with pinned host buffers (mixed form)
    m2 = api.build_model(cfg, form="mixed", device=local)
    s = torch.from_numpy(np.ascontiguousarray(M["th0"])).pin_memory().numpy()
    for _ in range(args.warmup):
        s = m2.step(s, api.production_dt(m2, s))
    sp = torch.empty((m2.Nk, m2.Nz), dtype=torch.complex128).pin_memory().numpy()
    sp[...] = s
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        dt = api.production_dt(m2, sp)
        out = m2.step(sp, dt)
        sp[...] = out
    el = time.perf_counter() - t0
    el = max_over_ranks(el)
    e2e = {"value": world * args.steps / el, "unit": "steps/s",
           "h2d_bytes_per_step": 2 * n_c * 16, "d2h_bytes_per_step": n_c * 16 + 8}

    # the batched form (the ensemble workload, a bounded sample of it): the
    # first B runs of the seeded 256-run list (uneven grids, models, Ra and
    # viscosity contrast), S steps each, in one native call -- mixed form
    # with the batched engine vs the FP64 plain form, both with the same host
    # concurrency; states resident in HBM, device synchronised on both sides
    batched = None
    if not args.no_batched:
        import collections

        from specmc_gb300 import ensemble
        runs = ensemble.ensemble_configs(256, seed=0)[:args.batch_runs]
        ensemble.march_ensemble_native(runs[:4], nsteps=2, concurrency=4, device=local,
                                       keep_states=False)                      # warm-up
        out = {}
        for form in ("mixed", "plain"):
            if form == "plain" and args.no_plain:
                continue
            torch.cuda.synchronize()
            res = ensemble.march_ensemble_native(runs, nsteps=args.batch_steps, form=form,
                                                 concurrency=args.batch_concurrency,
                                                 batched=(form == "mixed"), device=local,
                                                 keep_states=False)
            torch.cuda.synchronize()
            tm = res[0]["_timing"]
            nst = sum(r["steps"] for r in res)
            out[form] = dict(value=world * nst / tm["wall_s"], steps=nst, wall_s=tm["wall_s"],
                             status=dict(collections.Counter(r["status"] for r in res)),
                             batch_launches=tm["batch_launches"], batch_solves=tm["batch_solves"],
                             ctas_per_launch=(tm["batch_ctas"] / tm["batch_launches"]
                                              if tm["batch_launches"] else None))
        batched = {
            "metric": "aggregate steps/s of independent runs (batched ensemble sample)",
            "unit": "steps/s", "value": out["mixed"]["value"],
            "sample": "the first %d runs of the seeded 256-run ensemble (grids 32x24..128x96, "
                      "const/eta_z/eta_T, Ra 1e4..1e6, deta_T 1..1e4), %d steps each"
                      % (len(runs), args.batch_steps),
            "mixed_batched": out["mixed"], "plain": out.get("plain"),
            "batched_vs_plain": (out["mixed"]["value"] / out["plain"]["value"]
                                 if out.get("plain") else None),
            "concurrency": args.batch_concurrency}

    # roofline of the dominant kernel of the headline (mixed) form: the leaf
    # profile region with the largest share of the timed steps (aggregates
    # "step.*" / the memoised Stokes bracket and the engine's per-phase
    # sub-slots "name.phase" are not kernels)
    peaks, psrc = _peaks()
    prof = M["prof"]
    leaves = [p for p in prof if not p["name"].startswith("step.") and "." not in p["name"]
              and p["name"] != "stokes_memo_check"]
    dom = max(leaves, key=lambda p: p["ms"]) if leaves else None
    roof = None
    if dom is not None:
        avg_ms = dom["ms"] / max(dom["launches"], 1)
        per_launch = dom["work"] / max(dom["launches"], 1)
        if dom["is_bytes"]:
            ach = per_launch / (avg_ms / 1e3) / 1e9
            roof = {"bound": "hbm", "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                    "frac": ach / peaks["hbm_gbs"],
                    "traffic": DRAM_BYTES_PER_LAUNCH.get(dom["name"]),
                    "traffic_source": TRAFFIC_SOURCE,
                    "algorithmic_bytes_per_launch": per_launch,
                    "peak_source": psrc + ", copy bandwidth (of measured)"}
        else:
            ach = per_launch / (avg_ms / 1e3) / 1e12
            fp64 = 1.196
            roof = {"bound": "fp64", "achieved": ach, "peak": fp64, "unit": "TFLOP/s",
                    "frac": ach / fp64, "traffic": DRAM_BYTES_PER_LAUNCH.get(dom["name"]),
                    "peak_source": "FP64 FMA throughput measured on this pool's GB300 "
                                   "(1.196 TFLOP/s; no FP64 figure in MEASURED_PEAKS.json)"}
        roof["kernel"] = dom["name"]
        roof["launch_ms"] = avg_ms
        roof["share_of_timed"] = dom["ms"] / M["ms"]
    acc = None
    if P is not None:
        acc = {k: abs(M["diag"][k] - P["diag"][k]) / abs(P["diag"][k]) for k in ("Nu_top", "urms")}
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": M["ms"] / args.steps,
        # spread of the timed steps (the step is launch-bound, so load on the
        # shared host cores shows here first)
        "step_ms": {"min": M["step_ms"][0], "median": M["step_ms"][len(M["step_ms"]) // 2],
                    "max": M["step_ms"][-1]},
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        # the mixed form: FP32 (and double-float) inner Krylov iterations,
        # FP64 residuals, solution updates, factorisations and reductions
        "dtype": "fp32/fp64 mixed",
        "data": "synthetic (seeded conductive perturbation, random-free)",
        "config": dict(workload="eta_T 64x96 Ra=1e4 deta_T=1e3, 200-step adaptive march",
                       sample="steps %d..%d" % (args.warmup + 1, args.warmup + args.steps),
                       form="mixed (BFBT-FGMRES Stokes, explicit per-k inverse preconditioners)",
                       l2="flushed between timed steps (256 MiB write)",
                       parallelism="replicas" if world > 1 else "single", **WORKLOAD),
        "e2e": e2e, "gpu_launches": M["launches"], "roofline": roof, "cpu_baseline": cpu,
        "clocks": clk,
        "plain_fp64": None if P is None else {
            "value": world * args.steps / (P["ms"] / 1e3), "unit": "steps/s",
            "ms_per_step": P["ms"] / args.steps, "gpu_launches": P["launches"]},
        "mixed_vs_plain_rel_err": acc,
        "diag_after": {k: M["diag"][k] for k in ("Nu_top", "urms")},
        "kernel_regions": [dict(p, ms_per_step=p["ms"] / args.steps) for p in R["prof"]],
        "kernel_regions_ms_per_step": R["ms"] / args.steps,
        "batched": batched,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--cpu-steps", type=int, default=None,
                    help="CPU baseline: timed steps after the warm-up (default: --steps, at most 20)")
    ap.add_argument("--ref-steps", type=int, default=None,
                    help="reference arm: timed steps (default: --steps)")
    ap.add_argument("--ref-warmup", type=int, default=None,
                    help="reference arm: warm-up steps (default: --warmup)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-ensemble leg")
    ap.add_argument("--batch-runs", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=20)
    ap.add_argument("--batch-concurrency", type=int, default=16)
    ap.add_argument("--phases", action="store_true",
                    help="add the Krylov engine's per-phase times to kernel_regions")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if world > 1:
        import torch
        torch.distributed.init_process_group(
            "nccl", init_method="env://", world_size=world, rank=rank)
    rc = run_ours(args, rank, world)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
