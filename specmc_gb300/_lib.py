"""Build and load ``libspecmc_gb300.so`` (the C ABI of include/specmc_gb300.h).

The library is compiled in-tree with nvcc for sm_103a only.  There is no
fallback: if the shared library is missing or fails to load, every model
constructor raises.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(HERE, "libspecmc_gb300.so")
SOURCES = ("smc_spectral.cu", "smc_dense.cu", "smc_schur.cu", "smc_krylov.cu",
           "smc_pseudo.cu", "smc_fastops.cu", "smc_engine.cu", "smc_noalloc.cu", "smc_tala.cu", "smc_batch.cu", "smc_tc.cu", "smc_tclu.cu",
           "smc_runtime.cu")
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
              "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", os.path.join(ROOT, "include")]

SMC_HOST, SMC_DEVICE = 0, 1
SMC_MODEL_CONST, SMC_MODEL_ETA_Z, SMC_MODEL_ETA_T = 0, 1, 2
SMC_PRECOND_LEGACY, SMC_PRECOND_BFBT = 0, 1
SMC_FP64, SMC_MIXED = 0, 1
SMC_BOUSSINESQ, SMC_TALA = 0, 1
SMC_GRID, SMC_COEFFS, SMC_SYNTH_PAD, SMC_TRUNC_PAD = 0, 1, 2, 3
SMC_ABI_VERSION = 3


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    raise RuntimeError("nvcc not found")


def build(force=False, verbose=False):
    """Compile the CUDA sources (in parallel) and link the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    hdrs.append(os.path.join(ROOT, "include", "specmc_gb300.h"))
    newest_hdr = max(os.path.getmtime(h) for h in hdrs)

    def compile_one(src):
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        if (not force and os.path.exists(o)
                and os.path.getmtime(o) >= max(os.path.getmtime(s), newest_hdr)):
            return o
        cmd = [nvcc, *NVCC_FLAGS, "-c", s, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s" % (src, r.stderr))
        if verbose and r.stderr.strip():
            print(r.stderr)
        return o

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if (force or not os.path.exists(LIB_PATH)
            or os.path.getmtime(LIB_PATH) < max(os.path.getmtime(o) for o in objs)):
        cmd = [nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", *objs,
               "-o", LIB_PATH]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s" % r.stderr)
    return LIB_PATH


class SmcConfig(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_int), ("model", ctypes.c_int),
        ("Nx", ctypes.c_int), ("Nz", ctypes.c_int),
        ("Ra", ctypes.c_double), ("Lx", ctypes.c_double), ("deta_T", ctypes.c_double),
        ("internal_heating", ctypes.c_double), ("dissipation_number", ctypes.c_double),
        ("eta_min", ctypes.c_double), ("eta_max", ctypes.c_double),
        ("eta_smooth", ctypes.c_double), ("arrhenius_Ts", ctypes.c_double),
        ("precond", ctypes.c_int), ("symmetrize", ctypes.c_int),
        ("lag", ctypes.c_int), ("K", ctypes.c_int), ("max_K", ctypes.c_int),
        ("defect_tol", ctypes.c_double), ("eta_drift_tol", ctypes.c_double),
        ("stokes_rtol", ctypes.c_double), ("theta_rtol", ctypes.c_double),
        ("theta_maxiter", ctypes.c_int), ("theta_restart", ctypes.c_int),
        ("stokes_restart", ctypes.c_int), ("stokes_maxiter", ctypes.c_int),
        ("precision", ctypes.c_int), ("device", ctypes.c_int),
        ("arrhenius_E", ctypes.c_double), ("arrhenius_V", ctypes.c_double),
        ("compressibility", ctypes.c_int),
    ]


class SmcDiag(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in
                ("Nu_top", "Nu_bot", "Nu_energy", "urms", "umax", "amp")]


COUNTER_FIELDS = (
    ("n_steps", "q"), ("n_stokes", "q"), ("n_memo_hits", "q"),
    ("n_refresh", "q"), ("n_defect", "q"), ("n_defect_failed", "q"),
    ("n_defect_double_fail", "q"),
    ("n_bfbt_solves", "q"), ("n_bfbt_iters", "q"), ("n_bfbt_rescue", "q"),
    ("n_bfbt_rescue_direct", "q"), ("n_bfbt_rescue_weak", "q"),
    ("n_clip_T", "q"), ("n_T_out_of_range", "q"), ("n_clip_eta", "q"),
    ("n_smooth_eta", "q"), ("n_clip_eta_proj", "q"), ("n_smooth_eta_proj", "q"),
    ("n_theta_nonconv", "q"), ("n_be_fallback", "q"), ("n_theta_solves", "q"),
    ("n_theta_iters", "q"), ("theta_last_iters", "q"), ("last_K", "q"),
    ("max_T_excursion", "d"), ("last_corr", "d"), ("theta_last_res", "d"),
    ("last_bfbt_true_res", "d"), ("sym_removed", "d"),
    ("n_kernel_launches", "q"),
)


class SmcCounters(ctypes.Structure):
    _fields_ = [(k, ctypes.c_longlong if t == "q" else ctypes.c_double)
                for k, t in COUNTER_FIELDS]


class SmcMarchInfo(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_longlong), ("t", ctypes.c_double), ("dt", ctypes.c_double)]


SMC_RUN_OK, SMC_RUN_AMPLITUDE, SMC_RUN_NONFINITE, SMC_RUN_ERROR = 0, 1, 2, 3
RUN_STATUS = {SMC_RUN_OK: "ok", SMC_RUN_AMPLITUDE: "amplitude", SMC_RUN_NONFINITE: "non-finite",
              SMC_RUN_ERROR: "error"}


class SmcRunResult(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_longlong), ("t", ctypes.c_double), ("dt", ctypes.c_double),
                ("amp0", ctypes.c_double), ("amp", ctypes.c_double), ("seconds", ctypes.c_double),
                ("status", ctypes.c_int), ("reserved", ctypes.c_int)]


#: every entry point include/specmc_gb300.h declares
EXPORTED = ("smc_config_defaults", "smc_create", "smc_destroy", "smc_step", "smc_cfl_dt",
            "smc_production_dt", "smc_march_adaptive", "smc_march", "smc_diagnostics",
            "smc_stokes", "smc_velocity", "smc_project_mirror", "smc_transform",
            "smc_eta_of", "smc_schur_matvec", "smc_reset_history", "smc_counters_get",
            "smc_shape", "smc_stream", "smc_last_error", "smc_set_state", "smc_get_state",
            "smc_advance", "smc_profile", "smc_profile_get", "smc_set_option",
            "smc_grid_noalloc", "smc_get_history", "smc_set_history", "smc_dissipation_eta",
            "smc_create_many", "smc_march_many", "smc_batch_stats")

_LIB = None


def load(path=None):
    """Load the library (once) and declare its signatures.  Raises if absent."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(
            "libspecmc_gb300.so is not built (%s); run specmc_gb300._lib.build() "
            "or __graft_entry__.build() -- there is no CPU fallback" % path)
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    vp, dp, i, d, ll = ctypes.c_void_p, P(ctypes.c_double), ctypes.c_int, ctypes.c_double, ctypes.c_longlong
    sig = {
        "smc_config_defaults": (None, [P(SmcConfig)]),
        "smc_create": (i, [P(SmcConfig), P(vp)]),
        "smc_destroy": (i, [vp]),
        "smc_step": (i, [vp, vp, vp, i, d]),
        "smc_cfl_dt": (i, [vp, vp, i, d, d, d, dp]),
        "smc_production_dt": (i, [vp, vp, i, d, d, dp]),
        "smc_march_adaptive": (i, [vp, vp, vp, i, d, d, d, ll, P(SmcMarchInfo)]),
        "smc_march": (i, [vp, vp, vp, i, d, ll]),
        "smc_diagnostics": (i, [vp, vp, i, P(SmcDiag)]),
        "smc_stokes": (i, [vp, vp, i, vp, vp]),
        "smc_velocity": (i, [vp, vp, i, vp, vp]),
        "smc_project_mirror": (i, [vp, vp, vp, i]),
        "smc_transform": (i, [vp, i, vp, vp, i]),
        "smc_eta_of": (i, [vp, vp, i, vp]),
        "smc_dissipation_eta": (i, [vp, vp, i, vp]),
        "smc_schur_matvec": (i, [vp, vp, vp, vp, i]),
        "smc_reset_history": (i, [vp]),
        "smc_get_history": (i, [vp, vp, vp, i, dp, P(i)]),
        "smc_set_history": (i, [vp, vp, vp, i, d, i]),
        "smc_counters_get": (i, [vp, P(SmcCounters)]),
        "smc_shape": (i, [vp, P(ctypes.c_int), P(ctypes.c_int), P(ctypes.c_int), P(ctypes.c_int)]),
        "smc_stream": (vp, [vp]),
        "smc_last_error": (ctypes.c_char_p, []),
        "smc_set_state": (i, [vp, vp, i]),
        "smc_get_state": (i, [vp, vp, i]),
        "smc_advance": (i, [vp, d, ll, d, d, P(SmcMarchInfo)]),
        "smc_profile": (i, [vp, i]),
        "smc_set_option": (i, [vp, ctypes.c_char_p, d]),
        "smc_grid_noalloc": (i, [vp, vp, i, i, i, vp]),
        "smc_profile_get": (i, [vp, i, P(ctypes.c_char_p), dp, P(ll), dp, P(i)]),
        "smc_create_many": (i, [P(SmcConfig), i, P(vp)]),
        "smc_march_many": (i, [P(vp), i, ll, d, d, d, i, i, i, P(SmcRunResult)]),
        "smc_batch_stats": (i, [i, P(ll), P(ll), P(ll)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(rc):
    """Raise the library's last error for a negative return code."""
    if rc < 0:
        msg = _LIB.smc_last_error().decode() if _LIB is not None else "?"
        raise RuntimeError("specmc_gb300: " + msg)
    return rc
