"""Small, named workloads for profiling captures (ncu) of this package's kernels.

    python -m specmc_gb300.profile_workloads <name>

headline   the mixed form on eta_T 64x96 (deta_T 1e3, Ra 1e4, seed amp 3e-2): 6 CFL steps with
           the FP64 SIMT z-contractions, 6 with the tensor-core ones, then the first 8 runs of
           the seeded 256-run ensemble, 3 steps each, through the batched engine
ensemble   the first 8 runs of the seeded ensemble, 3 steps each, batched engine with refill off
           (each cooperative launch a fixed set of solves)
plain_lu   the plain form on eta_T 32x24, 64x48, 64x96 and 128x96, 4 steps each, with the dense
           Schur LU's trailing update in FP64 SIMT and on the tensor cores (prints the
           factorisation times)
"""
from __future__ import annotations

import ctypes
import sys
import time


def _eta_t(Nx, Nz):
    from .config import ConvectionConfig
    return ConvectionConfig(viscosity_model="eta_T", deta_T=1000.0, Ra=1e4, Nx=Nx, Nz=Nz)


def headline(steps=6):
    from . import _lib, api, ensemble
    for tc in (0.0, 1.0):
        m = api.build_model(_eta_t(64, 96), form="mixed")
        _lib.check(m._lib.smc_set_option(m._h, b"tc_transforms", tc))
        s = m.seed(amp=3e-2, m=1, n=1)
        for _ in range(steps):
            s = m.step(s, api.production_dt(m, s))
        print("tc_transforms", tc, "Nu_top", m.diagnostics(s)["Nu_top"])
        m.close()
    runs = ensemble.ensemble_configs(256, seed=0)[:8]
    res = ensemble.march_ensemble_native(runs, nsteps=3, concurrency=8, keep_states=False)
    print("ensemble", res[0]["_timing"])


def ensemble_fixed():
    from . import _lib, api, ensemble
    runs = ensemble.ensemble_configs(256, seed=0)[:8]
    h = api.build_model(runs[0]["cfg"], form="mixed")
    _lib.check(h._lib.smc_set_option(h._h, b"engine_batch_refill", 0.0))
    res = ensemble.march_ensemble_native(runs, nsteps=3, concurrency=8, keep_states=False)
    _lib.check(h._lib.smc_set_option(h._h, b"engine_batch_refill", 1.0))
    h.close()
    print("ensemble", res[0]["_timing"])


def plain_lu(steps=4):
    from . import _lib, api
    for Nx, Nz in ((32, 24), (64, 48), (64, 96), (128, 96)):
        for tc in (0.0, 1.0):
            m = api.build_model(_eta_t(Nx, Nz), form="plain")
            lib = m._lib
            _lib.check(lib.smc_set_option(m._h, b"tc_lu", tc))
            _lib.check(lib.smc_profile(m._h, 1))
            s = m.seed(amp=3e-2, m=1, n=1)
            t0 = time.time()
            for _ in range(steps):
                s = m.step(s, api.production_dt(m, s))
            el = time.time() - t0
            name, ms, nl = ctypes.c_char_p(), ctypes.c_double(), ctypes.c_longlong()
            work, isb = ctypes.c_double(), ctypes.c_int()
            lu = None
            for slot in range(64):
                _lib.check(lib.smc_profile_get(m._h, slot, ctypes.byref(name), ctypes.byref(ms),
                                               ctypes.byref(nl), ctypes.byref(work), ctypes.byref(isb)))
                if not name.value:
                    break
                if name.value == b"schur_lu":
                    lu = (ms.value, nl.value)
            print("%dx%d tc_lu %d: %d steps %.3f s, schur_lu (ms, launches) %s, Nu_top %.12f"
                  % (Nx, Nz, tc, steps, el, lu, m.diagnostics(s)["Nu_top"]), flush=True)
            m.close()


WORKLOADS = {"headline": headline, "ensemble": ensemble_fixed, "plain_lu": plain_lu}

if __name__ == "__main__":
    from . import _lib
    _lib.build()
    name = sys.argv[1] if len(sys.argv) > 1 else ""
    if name not in WORKLOADS:
        sys.exit("usage: python -m specmc_gb300.profile_workloads {%s}" % ",".join(WORKLOADS))
    WORKLOADS[name]()
