"""The C-ABI boundary without a GPU: the library builds, loads and exports
every symbol include/specmc_gb300.h declares; the host mirror of the
reference interface validates like the reference."""
import os
import re
import warnings

import numpy as np
import pytest

from conftest import ROOT


def test_library_exports_every_declared_symbol():
    from specmc_gb300 import _lib
    _lib.build()
    lib = _lib.load()
    hdr = open(os.path.join(ROOT, "include", "specmc_gb300.h")).read()
    declared = set(re.findall(r"^(?:int|void\s*\*?|const char\s*\*)\s*(smc_[a-z_]+)\s*\(",
                              hdr, flags=re.M))
    assert declared, "no declarations found"
    assert declared == set(_lib.EXPORTED)
    for name in declared:
        assert hasattr(lib, name), name


def test_config_defaults_roundtrip():
    import ctypes
    from specmc_gb300 import _lib
    lib = _lib.load()
    c = _lib.SmcConfig()
    lib.smc_config_defaults(ctypes.byref(c))
    assert (c.Nx, c.Nz, c.lag, c.K, c.max_K) == (64, 96, 16, 3, 8)
    assert c.defect_tol == 1e-8 and c.theta_rtol == 1e-10 and c.stokes_rtol == 1e-8
    assert c.theta_restart == 40 and c.stokes_restart == 80 and c.stokes_maxiter == 800


BAD_CONFIGS = [
    (dict(Nx=3), b"Nx"),
    (dict(Nx=30, Nz=3), b"Nx, Nz"),
    (dict(Nx=34 + 1), b"even"),
    (dict(abi_version=1), b"abi_version"),
    (dict(model=7), b"unknown model"),
    (dict(Ra=-1.0), b"positive"),
    (dict(eta_min=2.0, eta_max=1.0), b"eta window"),
    (dict(lag=0), b"defect-correction"),
    (dict(theta_restart=0), b"restart"),
    (dict(precision=5), b"precision"),
    (dict(arrhenius_V=-1.0), b"arrhenius_V"),
    (dict(arrhenius_V=0.5, arrhenius_Ts=0.0), b"pV law"),
    (dict(compressibility=4), b"compressibility"),
    (dict(compressibility=1, dissipation_number=-0.5), b"dissipation_number"),
    (dict(compressibility=1, precision=1), b"FP64 form only"),
    (dict(compressibility=1, precond=1), b"Boussinesq-only"),
]


@pytest.mark.parametrize("fields,msg", BAD_CONFIGS)
def test_create_reports_errors_not_crashes(fields, msg):
    """A bad config is a hard error with a message, raised before any device
    work (no GPU needed)."""
    import ctypes
    from specmc_gb300 import _lib
    lib = _lib.load()
    c = _lib.SmcConfig()
    lib.smc_config_defaults(ctypes.byref(c))
    for k, v in fields.items():
        setattr(c, k, v)
    h = ctypes.c_void_p()
    assert lib.smc_create(ctypes.byref(c), ctypes.byref(h)) < 0
    assert msg in lib.smc_last_error(), lib.smc_last_error()
    assert not h.value


def test_config_validation_mirrors_reference():
    from specmc_gb300.config import ConvectionConfig
    with pytest.raises(ValueError):
        ConvectionConfig(viscosity_model="nope")
    with pytest.raises(NotImplementedError):
        ConvectionConfig(viscosity_model="eta_Tz")
    with pytest.raises(ValueError):
        ConvectionConfig(viscosity_model="eta_T", arrhenius_Ts=1.0)
    with pytest.raises(ValueError):
        ConvectionConfig(eta_min=1.0, eta_max=0.5)
    with pytest.raises(ValueError):
        ConvectionConfig(precond="ilu")
    with pytest.raises(ValueError):
        ConvectionConfig(K=9)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        ConvectionConfig(symmetrize=False)
        assert any(issubclass(x.category, UserWarning) for x in w)
    c = ConvectionConfig(viscosity_model="arrhenius", arrhenius_Ts=1.0)
    assert c.canonical()["viscosity_model"] == "arrhenius"


def test_pv_config_and_calibration():
    """The pressure-dependent Arrhenius branch (arrhenius_V > 0): the
    reference's validation rules (specmc/config.py:496-560) and its
    calibration (physics/reference_state.py:277-364), pinned against the
    reference's own values (tests/golden/pv_calibration.npz)."""
    import os
    from specmc_gb300.config import ConvectionConfig, arrhenius_effective_E
    from specmc_gb300.reference_state import calibrate_pv
    ConvectionConfig(viscosity_model="arrhenius", arrhenius_V=2.0)
    ConvectionConfig(viscosity_model="arrhenius", arrhenius_V=2.0, reference_anchor="Ea")
    ok = calibrate_pv(anchor="D", V=2.0, deta_T=1000.0)
    ConvectionConfig(viscosity_model="arrhenius", arrhenius_V=2.0, arrhenius_Ts=ok["Ts"], arrhenius_E=ok["E"])
    for bad in (dict(viscosity_model="arrhenius", arrhenius_V=2.0, reference_anchor="X"),
                dict(viscosity_model="eta_T", arrhenius_V=2.0),
                dict(viscosity_model="arrhenius", arrhenius_V=2.0, arrhenius_Ts=0.5),
                dict(viscosity_model="arrhenius", arrhenius_V=2.0, arrhenius_E=1.0),
                dict(viscosity_model="arrhenius", arrhenius_V=-1.0)):
        with pytest.raises(ValueError):
            ConvectionConfig(**bad)
    assert arrhenius_effective_E(ConvectionConfig(viscosity_model="arrhenius", arrhenius_V=2.0)) == ok["E"]
    rows = np.load(os.path.join(os.path.dirname(__file__), "golden", "pv_calibration.npz"))["rows"]
    for a, V, D, E, Vt, Ts, C, lnD in rows:
        r = calibrate_pv(anchor="Ea" if a == 0 else "D", V=None if V < 0 else V,
                         deta_T=None if D < 0 else D)
        assert (r["E"], r["V"], r["Ts"], r["C"], r["ln_D"]) == (E, Vt, Ts, C, lnD)


def test_api_dispatch_table():
    from specmc_gb300 import api
    from specmc_gb300.config import ConvectionConfig
    from specmc_gb300.solver import RBC, RBCCoupled, RBCImplicitTheta
    assert api.MODEL_CLASSES == {"const": RBC, "eta_z": RBCImplicitTheta,
                                 "eta_T": RBCCoupled, "arrhenius": RBCCoupled}
    d = api.describe(ConvectionConfig())
    assert d["model_class"] == "RBCCoupled" and d["numerics"]["DTMAX"] == 4e-5
    spec = api.model_spec(ConvectionConfig(defect_tol=0.0, K=3))
    assert spec["kwargs"]["defect_tol"] is None
    tala = ConvectionConfig(compressibility="tala", precond="legacy", dissipation_number=0.5)
    assert api.model_spec(tala)["kwargs"]["compressibility"] == "tala"
    # the TALA route is the FP64 form's: the mixed form refuses it before any
    # device work
    with pytest.raises(NotImplementedError):
        api.build_model(tala, form="mixed")


def test_config_and_model_spec_match_reference_on_seeded_cases():
    """ConvectionConfig and api.model_spec against the reference on 300 seeded
    configurations (tests/golden/config_cases.json, written by the reference's
    own ConvectionConfig / api.model_spec): the same outcome (valid, ValueError,
    NotImplementedError), the same warnings, the same canonical() and the same
    model / builder / constructor kwargs and api.describe(), TALA included."""
    import json
    from specmc_gb300 import api
    from specmc_gb300.config import ConvectionConfig
    with open(os.path.join(os.path.dirname(__file__), "golden", "config_cases.json")) as f:
        cases = json.load(f)
    assert len(cases) == 300
    for c in cases:
        with warnings.catch_warnings(record=True) as w:
            warnings.simplefilter("always")
            try:
                cfg = ConvectionConfig(**c["kw"])
                outcome = "ok"
            except Exception as ex:                      # noqa: BLE001 -- the class is compared
                outcome, cfg = type(ex).__name__, None
        assert outcome == c["outcome"], c["kw"]
        assert sorted({x.category.__name__ for x in w}) == c["warnings"], c["kw"]
        if cfg is None:
            continue
        assert cfg.canonical() == c["canonical"], c["kw"]
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")            # validate() repeats the warnings above
            sp = api.model_spec(cfg)
            d = json.loads(json.dumps(api.describe(cfg), default=str))
        assert (sp["model"], sp["builder"], sp["kwargs"]) == (
            c["spec"]["model"], c["spec"]["builder"], c["spec"]["kwargs"]), c["kw"]
        assert d == c["describe"], c["kw"]


def test_model_basis_attributes_match_reference():
    """The host copies the GPU models expose (x, z, kx, V, Vi, D, wq) equal the
    reference's RBC attributes (tests/golden/transforms_16x12.npz)."""
    from specmc_gb300.solver import basis_arrays
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "transforms_16x12.npz"))
    b = basis_arrays(16, 12, 2.0)
    for k in ("x", "z", "kx", "V", "Vi", "D", "wq"):
        ref = g[k]
        assert b[k].shape == ref.shape, k
        assert np.max(np.abs(b[k] - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref))), k


def test_header_is_plain_c_and_a_c_caller_links(tmp_path):
    """include/specmc_gb300.h compiles as C99 and a C caller links against
    libspecmc_gb300.so; the program runs the calls that need no GPU (the
    defaults and a rejected configuration with its message)."""
    import shutil
    import subprocess
    from specmc_gb300 import _lib
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    _lib.build()
    src = tmp_path / "caller.c"
    src.write_text(r'''
#include <stdio.h>
#include <string.h>
#include "specmc_gb300.h"
int main(void) {
  smc_config c;
  smc_handle* h = 0;
  smc_config_defaults(&c);
  if (c.abi_version != SMC_ABI_VERSION || c.Nx != 64 || c.Nz != 96) return 2;
  c.compressibility = SMC_TALA;
  c.precision = SMC_MIXED;
  if (smc_create(&c, &h) >= 0 || h != 0) return 3;
  if (!strstr(smc_last_error(), "FP64 form only")) return 4;
  printf("ok %s\n", smc_last_error());
  return 0;
}
''')
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = tmp_path / "caller"
    subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-L", libdir, "-lspecmc_gb300", "-o", str(exe)], check=True)
    env = dict(os.environ, LD_LIBRARY_PATH=libdir + os.pathsep + os.environ.get("LD_LIBRARY_PATH", ""))
    out = subprocess.run([str(exe)], env=env, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)
    assert out.stdout.startswith("ok ")


def test_ctypes_mirrors_match_the_c_structs(tmp_path):
    """Every field of the Python mirrors of smc_config, smc_diag,
    smc_counters, smc_march_info and smc_run_result sits at the offset the C compiler gives
    it, and the structs have the same size (a mismatch would silently corrupt
    every call)."""
    import ctypes
    import shutil
    import subprocess
    from specmc_gb300 import _lib
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    mirrors = {"smc_config": _lib.SmcConfig, "smc_diag": _lib.SmcDiag,
               "smc_counters": _lib.SmcCounters, "smc_march_info": _lib.SmcMarchInfo,
               "smc_run_result": _lib.SmcRunResult}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "specmc_gb300.h"',
             'int main(void) {']
    for cname, py in mirrors.items():
        lines.append('  printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    c = {}
    for line in out:
        if line:
            cname, field, value = line.split()
            c[(cname, field)] = int(value)
    for cname, py in mirrors.items():
        assert ctypes.sizeof(py) == c[(cname, "sizeof")], cname
        for fname, _ in py._fields_:
            assert getattr(py, fname).offset == c[(cname, fname)], (cname, fname)
