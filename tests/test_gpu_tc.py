"""The tensor-core z-contractions (tcgen05, bf16 slices with exact FP32
accumulation in tensor memory, FP64 result; option "tc_transforms") against
the FP64 SIMT contractions and the oracle's NumPy transforms."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def gb():
    from specmc_gb300 import _lib
    _lib.build()
    import specmc_gb300.api as api
    from specmc_gb300.config import ConvectionConfig
    return api, ConvectionConfig, _lib


def _transforms(m, lib, cf, g, gp):
    out = {}
    for name, kind, src, shape in (("grid", lib.SMC_GRID, cf, (m.Nx, m.Nz)),
                                   ("coeffs", lib.SMC_COEFFS, g, (m.Nk, m.Nz)),
                                   ("synth_pad", lib.SMC_SYNTH_PAD, cf, (2 * m.Nx, m.Nz)),
                                   ("trunc_pad", lib.SMC_TRUNC_PAD, gp, (m.Nk, m.Nz))):
        dt = np.complex128 if name in ("coeffs", "trunc_pad") else np.float64
        o = np.empty(shape, dtype=dt)
        s = np.ascontiguousarray(src)
        lib.check(m._lib.smc_transform(m._h, kind, s.ctypes.data_as(ctypes.c_void_p),
                                       o.ctypes.data_as(ctypes.c_void_p), lib.SMC_HOST))
        out[name] = o
    return out


@pytest.mark.parametrize("Nx,Nz", [(16, 12), (32, 24), (64, 96), (128, 96), (64, 128)])
def test_tc_transforms_match_fp64(gb, Nx, Nz):
    """grid / coeffs / padded synthesis on the tensor cores agree with the
    FP64 SIMT contractions and with the oracle to FP64 roundoff (1e-13 of the
    largest value; the SIMT contraction's own rounding is ~N 2^-53)."""
    from oracle import specmc_oracle as O
    api, CC, lib = gb
    cfg = CC(viscosity_model="const", Nx=Nx, Nz=Nz)
    m_tc, m_64 = api.build_model(cfg), api.build_model(cfg)
    lib.check(m_tc._lib.smc_set_option(m_tc._h, b"tc_transforms", 1.0))
    o = O.build(cfg)
    rng = np.random.default_rng(Nx * 1000 + Nz)
    # coefficients that decay like a smooth field's
    cf = (rng.standard_normal((m_tc.Nk, Nz)) + 1j * rng.standard_normal((m_tc.Nk, Nz)))
    cf /= (1.0 + np.arange(m_tc.Nk))[:, None] * (1.0 + np.arange(Nz))[None, :]
    g = rng.standard_normal((Nx, Nz))
    gp = rng.standard_normal((2 * Nx, Nz))
    a = _transforms(m_tc, lib, cf, g, gp)
    b = _transforms(m_64, lib, cf, g, gp)
    ref = dict(grid=o.grid(cf), coeffs=o.coeffs(g), synth_pad=o.synth_pad(cf),
               trunc_pad=o.trunc_pad(gp))
    for k in a:
        print("%dx%d %-9s tc-simt %.2e  tc-oracle %.2e  simt-oracle %.2e"
              % (Nx, Nz, k, _rel(a[k], b[k]), _rel(a[k], ref[k]), _rel(b[k], ref[k])))
        assert _rel(a[k], b[k]) < 1e-13, (k, _rel(a[k], b[k]))
        assert _rel(a[k], ref[k]) < 1e-13, (k, _rel(a[k], ref[k]))
    m_tc.close()
    m_64.close()


def test_tc_mixed_march_matches_simt(gb):
    """The mixed form on the headline grid with the tensor-core contractions
    equals the same march with FP64 SIMT contractions to 1e-9 in Nu and Vrms
    after 20 steps (both sit at FP64 roundoff of the same operators)."""
    api, CC, lib = gb
    cfg = CC(viscosity_model="eta_T", deta_T=1000.0, Ra=1e4, Nx=64, Nz=96)
    out = {}
    for tc in (0.0, 1.0):
        m = api.build_model(cfg, form="mixed")
        lib.check(m._lib.smc_set_option(m._h, b"tc_transforms", tc))
        s = m.seed(amp=3e-2, m=1, n=1)
        for _ in range(20):
            s = m.step(s, api.production_dt(m, s))
        out[tc] = m.diagnostics(s)
        m.close()
    for key in ("Nu_top", "urms", "Nu_energy"):
        assert abs(out[1.0][key] - out[0.0][key]) <= 1e-9 * abs(out[0.0][key]), key


def _cfg_kw(g):
    return {k[4:]: g[k].item() for k in g.files if k.startswith("cfg_")}


@pytest.mark.parametrize("case", ["march_etaT_32x24.npz", "march_etaT_64x96.npz"])
def test_tc_lu_plain_march_matches_reference(gb, case):
    """The plain form with the dense Schur LU's trailing updates on the tensor
    cores (option "tc_lu") against the reference's own march records: the
    same bars as the FP64 SIMT LU (state 1e-7, Nu / Vrms 1e-8) and the same
    refresh and defect-correction counts (the 32x24 march refreshes its
    factor 24 times in 25 steps)."""
    import os
    from conftest import GOLDEN
    api, CC, lib = gb
    g = np.load(os.path.join(GOLDEN, case))
    m = api.build_model(CC(**_cfg_kw(g)))
    lib.check(m._lib.smc_set_option(m._h, b"tc_lu", 1.0))
    s = np.array(g["that0"], copy=True)
    worst = 0.0
    for n in range(len(g["dts"])):
        dt = api.production_dt(m, s)
        assert abs(dt - g["dts"][n]) <= 1e-9 * g["dts"][n]
        s = m.step(s, dt)
        worst = max(worst, _rel(s, g["states"][n]))
    assert worst < 1e-7, worst
    d = m.diagnostics(s)
    for key in ("Nu_top", "urms"):
        ref = g["diag_" + key].item()
        assert abs(d[key] - ref) <= 1e-8 * abs(ref), (key, d[key], ref)
    c = m.counters()
    for key in ("n_refresh", "n_defect", "n_defect_failed"):
        assert c[key] == int(g["ctr_" + key]), (key, c[key])
    m.close()
