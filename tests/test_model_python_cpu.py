"""The Python layer of the GPU models on the CPU: a stand-in for the
library's device calls (smc_create hands out a handle, the counters and
dissipation_eta answer with fixed values) lets the code that runs after a
successful smc_create execute here -- the reference-named attributes of the
TALA reference state, describe(), the theta view and the parsing of
dissipation_eta's result.  The real library fills the config defaults."""
import ctypes

import numpy as np
import pytest


class _FakeLib:
    def __init__(self, real, rows):
        self._real, self.rows, self.created, self.destroyed = real, rows, [], 0

    def smc_config_defaults(self, cfg):
        return self._real.smc_config_defaults(cfg)

    def smc_create(self, cfg_ref, h_ref):
        self.created.append(ctypes.cast(cfg_ref, ctypes.POINTER(type(cfg_ref._obj))).contents)
        h_ref._obj.value = 1
        return 0

    def smc_destroy(self, h):
        self.destroyed += 1
        return 0

    def smc_counters_get(self, h, ref):
        ref._obj.theta_last_iters, ref._obj.n_theta_solves = 7, 3
        return 0

    def smc_dissipation_eta(self, h, buf, mem, rows_ref):
        rows_ref._obj.value = self.rows
        if self.rows:
            n = 16 * 12 if self.rows > 1 else 12
            arr = np.ctypeslib.as_array(ctypes.cast(buf, ctypes.POINTER(ctypes.c_double)), (n,))
            arr[:] = np.arange(n, dtype=float) + 1.0
        return 0


@pytest.fixture()
def fake(monkeypatch):
    from specmc_gb300 import _lib
    real = _lib.load()

    def make(rows):
        f = _FakeLib(real, rows)
        monkeypatch.setattr(_lib, "load", lambda: f)
        return f
    return make


def test_tala_model_attributes_and_describe(fake):
    from specmc_gb300 import _lib, api, compressibility as C
    from specmc_gb300.config import ConvectionConfig
    f = fake(16)
    cfg = ConvectionConfig(Nx=16, Nz=12, viscosity_model="eta_T", compressibility="tala",
                           dissipation_number=0.7, precond="legacy")
    m = api.build_model(cfg)
    c = f.created[-1]
    assert c.compressibility == _lib.SMC_TALA and c.precision == _lib.SMC_FP64
    assert c.model == _lib.SMC_MODEL_ETA_T and abs(c.dissipation_number - 0.7) == 0.0
    assert m.tala_active and m.tala_a == -0.7 and m.tala_record["Di"] == 0.7
    assert np.array_equal(m.rho_grid, C.rho_bar_grid(m.z, 0.7))
    assert np.array_equal(m.rho2_c, C.rho_bar_coeffs(m.Vi, m.z, 1.4))
    d = m.describe()
    assert d["compressibility"] == "tala" and d["tala_active"] and d["theta_last_iters"] == 7
    assert m.theta.last_iters == 7 and m.theta.n_solves == 3 and m.theta.rtol == 1e-10
    eta = m.dissipation_eta()
    assert eta.shape == (16, 12) and eta[0, 0] == 1.0 and eta[-1, -1] == 16 * 12
    m.close()
    assert f.destroyed == 1


def test_boussinesq_model_and_dissipation_eta_shapes(fake):
    from specmc_gb300 import _lib, api
    from specmc_gb300.config import ConvectionConfig
    f = fake(1)
    m = api.build_model(ConvectionConfig(Nx=16, Nz=12, viscosity_model="eta_z", deta_T=100.0))
    assert f.created[-1].compressibility == _lib.SMC_BOUSSINESQ
    assert not m.tala_active and m.tala_a == 0.0 and m.rho_grid is None
    prof = m.dissipation_eta()
    assert prof.shape == (12,) and np.array_equal(prof, np.arange(12.0) + 1.0)
    f.rows = 0
    assert m.dissipation_eta() is None
    with pytest.raises(NotImplementedError):
        api.build_model(ConvectionConfig(Nx=16, Nz=12, compressibility="tala", precond="legacy"),
                        form="mixed")
