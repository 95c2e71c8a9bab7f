"""GPU model objects with the duck-typed contract of SpecMC's models.

``RBC`` (``specmc/core/rbc_galerkin.py:258``), ``RBCImplicitTheta``
(``specmc/core/implicit_theta.py:538``) and ``RBCCoupled``
(``specmc/models/coupled_model.py:123``) are thin handles over one native
model of ``libspecmc_gb300.so``: every step, Stokes solve, transform and
reduction runs on the GPU.  The Python side only moves the caller's arrays
across the C ABI and exposes the reference's attribute names (``x``, ``z``,
``kx``, ``V``, ``Vi``, ``D``, ``wq``, ``Nk`` ...) and counters.

State arrays are (Nk, Nz) complex128 Chebyshev-per-rfft-mode coefficients.
Arguments may be NumPy arrays (host) or CUDA torch tensors (device; the
result is then a CUDA tensor too).  ``step`` never writes its argument.
"""
from __future__ import annotations

import ctypes

import numpy as np
from numpy.polynomial import chebyshev as _npcheb

from . import _lib

__all__ = ["RBC", "RBCImplicitTheta", "RBCCoupled", "GpuModel", "ThetaSolverView"]


def _cgl(N):
    return 0.5 * (1.0 - np.cos(np.pi * np.arange(N) / (N - 1)))


def basis_arrays(Nx, Nz, Lx):
    """-> the host copies of the discretisation the model exposes under the
    reference's names (rbc_galerkin.py:63-81, :258-290): kx = 2 pi rfftfreq,
    x nodes, CGL nodes z (ascending), V (values = V @ coefficients, Chebyshev
    in 2z - 1), Vi = V^-1, the coefficient-space derivative D (d/dz on [0, 1])
    and the Clenshaw-Curtis weights wq."""
    Nx, Nz, Lx = int(Nx), int(Nz), float(Lx)
    z = _cgl(Nz)
    V = _npcheb.chebvander(2.0 * z - 1.0, Nz - 1)
    Vi = np.linalg.inv(V)
    D = np.zeros((Nz, Nz))
    for k in range(1, Nz):
        n = np.arange(k - 1, -1, -2)
        D[n, k] = 4.0 * k
        if n[-1] == 0:
            D[0, k] = 2.0 * k
    gk = np.array([0.0 if (k % 2) else 1.0 / (1.0 - k * k) for k in range(Nz)])
    gk[0] = 1.0
    return dict(kx=2 * np.pi * np.fft.rfftfreq(Nx, d=Lx / Nx), x=np.arange(Nx) * Lx / Nx, z=z,
                V=V, Vi=Vi, D=D, wq=Vi.T @ gk)


class GpuModel:
    """Common handle logic of the three model classes."""

    _MODEL = None

    def __init__(self, *, Ra=1e4, Nx=64, Nz=48, Lx=2.0, deta_T=1000.0,
                 internal_heating=0.0, dissipation_number=0.0, eta_min=1e-3,
                 eta_max=1e3, eta_smooth=0.0, arrhenius_Ts=0.0, arrhenius_E=0.0,
                 arrhenius_V=0.0, reference_anchor="D", precond="legacy",
                 symmetrize=True, lag=16, K=3, defect_tol=1e-8, max_K=8,
                 eta_drift_tol=0.1, stokes_rtol=1e-8, theta_rtol=1e-10,
                 theta_maxiter=200, theta_restart=40, stokes_restart=80,
                 stokes_maxiter=800, compressibility="boussinesq", device=0, form="plain",
                 **_ignored):
        from .config import normalize_compressibility
        comp = normalize_compressibility(compressibility)
        if comp not in ("boussinesq", "tala"):
            raise NotImplementedError("compressibility=%r is not implemented" % (compressibility,))
        if comp == "tala" and str(form).lower() == "mixed":
            raise NotImplementedError("compressibility='tala' runs the plain (FP64) form only")
        lib = _lib.load()
        c = _lib.SmcConfig()
        lib.smc_config_defaults(ctypes.byref(c))
        c.model = self._MODEL
        c.Nx, c.Nz = int(Nx), int(Nz)
        c.Ra, c.Lx, c.deta_T = float(Ra), float(Lx), float(deta_T)
        c.internal_heating = float(internal_heating)
        c.dissipation_number = float(dissipation_number)
        c.eta_min, c.eta_max = float(eta_min), float(eta_max)
        c.eta_smooth = float(eta_smooth)
        c.arrhenius_Ts = float(arrhenius_Ts)
        # the pressure-dependent Arrhenius law pV(L): Ts, E-tilde, V-tilde from
        # the one calibration (models/coupled_model.py:188-229)
        self.pv_record = None
        if float(arrhenius_V) > 0.0:
            from .reference_state import calibrate_pv
            anchor = str(reference_anchor)
            rec = calibrate_pv(anchor=anchor, V=float(arrhenius_V),
                               deta_T=(float(deta_T) if anchor == "D" else None))
            if float(arrhenius_Ts) != 0.0 and abs(float(arrhenius_Ts) - rec["Ts"]) > 1e-12 * rec["Ts"]:
                raise ValueError("arrhenius_Ts=%r contradicts the reference-state value Ts = %r"
                                 % (arrhenius_Ts, rec["Ts"]))
            if float(arrhenius_E) != 0.0 and abs(float(arrhenius_E) - rec["E"]) > 1e-12 * abs(rec["E"]):
                raise ValueError("arrhenius_E=%r contradicts the calibrated pV activation %r"
                                 % (arrhenius_E, rec["E"]))
            self.pv_record = rec
            c.arrhenius_Ts, c.arrhenius_E, c.arrhenius_V = rec["Ts"], rec["E"], rec["V"]
        c.precond = _lib.SMC_PRECOND_BFBT if str(precond).lower() == "bfbt" else _lib.SMC_PRECOND_LEGACY
        c.symmetrize = 1 if symmetrize else 0
        c.lag, c.K, c.max_K = int(lag), int(K), int(max_K)
        c.defect_tol = float(defect_tol) if defect_tol is not None else 0.0
        c.eta_drift_tol = float(eta_drift_tol)
        c.stokes_rtol, c.theta_rtol = float(stokes_rtol), float(theta_rtol)
        c.theta_maxiter, c.theta_restart = int(theta_maxiter), int(theta_restart)
        c.stokes_restart, c.stokes_maxiter = int(stokes_restart), int(stokes_maxiter)
        c.device = int(device)
        c.compressibility = _lib.SMC_TALA if comp == "tala" else _lib.SMC_BOUSSINESQ
        form = str(form).lower()
        if form not in ("plain", "mixed"):
            raise ValueError("form must be 'plain' (FP64, the reference algorithm) or "
                             "'mixed' (the fast form), got %r" % (form,))
        c.precision = _lib.SMC_MIXED if form == "mixed" else _lib.SMC_FP64
        self.form = form
        self._cfg = c
        self._lib = lib
        h = ctypes.c_void_p()
        _lib.check(lib.smc_create(ctypes.byref(c), ctypes.byref(h)))
        self._h = h
        self.Ra, self.Nx, self.Nz, self.Lx = float(Ra), int(Nx), int(Nz), float(Lx)
        self.deta_T = float(deta_T)
        self.internal_heating = float(internal_heating)
        self.dissipation_number = float(dissipation_number)
        for k, v in basis_arrays(self.Nx, self.Nz, self.Lx).items():
            setattr(self, k, v)
        self.Nk = len(self.kx)
        self.Np = 2 * self.Nx
        self.dealias = True
        # the TALA reference state under the reference's names
        # (core/rbc_galerkin.py:288-312); the library builds the same profiles
        self.compressibility = comp
        self.tala_active = comp == "tala"
        if self.tala_active:
            from . import compressibility as COMP
            Di = self.dissipation_number
            self.tala_a = COMP.a_coeff(Di)
            self.rho_grid = COMP.rho_bar_grid(self.z, Di)
            self.rho_c = COMP.rho_bar_coeffs(self.Vi, self.z, Di)
            self.rho2_c = COMP.rho_bar_coeffs(self.Vi, self.z, 2.0 * Di)
            self.tala_record = COMP.record(Di)
        else:
            self.tala_a = 0.0
            self.rho_grid = self.rho_c = self.rho2_c = self.tala_record = None

    # ------------------------------------------------------------ plumbing
    def close(self):
        if getattr(self, "_h", None):
            self._lib.smc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _is_device(a):
        return hasattr(a, "is_cuda") and bool(a.is_cuda)

    def _spec_in(self, that):
        """-> (pointer, mem, keepalive) for an (Nk, Nz) complex state."""
        if self._is_device(that):
            import torch
            t = that.to(torch.complex128).contiguous()
            if tuple(t.shape) != (self.Nk, self.Nz):
                raise ValueError("state must be (Nk, Nz) = (%d, %d)" % (self.Nk, self.Nz))
            # the library reads it on the handle's own stream: finish the
            # producer's work on the current torch stream first
            torch.cuda.current_stream(t.device).synchronize()
            return ctypes.c_void_p(t.data_ptr()), _lib.SMC_DEVICE, t
        a = np.ascontiguousarray(np.asarray(that), dtype=np.complex128)
        if a.shape != (self.Nk, self.Nz):
            raise ValueError("state must be (Nk, Nz) = (%d, %d), got %r" % (self.Nk, self.Nz, a.shape))
        return a.ctypes.data_as(ctypes.c_void_p), _lib.SMC_HOST, a

    def _spec_out(self, like_device):
        if like_device:
            import torch
            t = torch.empty((self.Nk, self.Nz), dtype=torch.complex128, device="cuda")
            return ctypes.c_void_p(t.data_ptr()), t
        a = np.empty((self.Nk, self.Nz), dtype=np.complex128)
        return a.ctypes.data_as(ctypes.c_void_p), a

    def _grid_out(self, Ng, like_device):
        if like_device:
            import torch
            t = torch.empty((Ng, self.Nz), dtype=torch.float64, device="cuda")
            return ctypes.c_void_p(t.data_ptr()), t
        a = np.empty((Ng, self.Nz), dtype=np.float64)
        return a.ctypes.data_as(ctypes.c_void_p), a

    # ---------------------------------------------------------- time step
    def step(self, that, dt):
        """One time step; returns the new state (the argument is not written)."""
        p, mem, keep = self._spec_in(that)
        q, out = self._spec_out(mem == _lib.SMC_DEVICE)
        _lib.check(self._lib.smc_step(self._h, p, q, mem, float(dt)))
        return out

    def cfl_dt(self, that, safety=0.5, dtmax=5e-3, dtmin=1e-10):
        p, mem, keep = self._spec_in(that)
        dt = ctypes.c_double()
        _lib.check(self._lib.smc_cfl_dt(self._h, p, mem, float(safety), float(dtmax),
                                        float(dtmin), ctypes.byref(dt)))
        return float(dt.value)

    def production_dt(self, that, safety=40.0, dtmax=4e-5):
        p, mem, keep = self._spec_in(that)
        dt = ctypes.c_double()
        _lib.check(self._lib.smc_production_dt(self._h, p, mem, float(safety), float(dtmax),
                                               ctypes.byref(dt)))
        return float(dt.value)

    def march_adaptive(self, that, tstop, safety=40.0, dtmax=4e-5, max_steps=0):
        p, mem, keep = self._spec_in(that)
        q, out = self._spec_out(mem == _lib.SMC_DEVICE)
        info = _lib.SmcMarchInfo()
        _lib.check(self._lib.smc_march_adaptive(self._h, p, q, mem, float(tstop), float(safety),
                                                float(dtmax), int(max_steps), ctypes.byref(info)))
        return out, dict(steps=int(info.steps), t=float(info.t), dt=float(info.dt))

    def march(self, that, dt, nsteps):
        p, mem, keep = self._spec_in(that)
        q, out = self._spec_out(mem == _lib.SMC_DEVICE)
        _lib.check(self._lib.smc_march(self._h, p, q, mem, float(dt), int(nsteps)))
        return out

    def reset_history(self):
        _lib.check(self._lib.smc_reset_history(self._h))

    def get_history(self):
        """-> dict(prev, psi_prev, dt_prev, have_prev): the BDF2 history of the
        temperature step (NumPy arrays)."""
        prev = np.empty((self.Nk, self.Nz), dtype=np.complex128)
        psi = np.empty_like(prev)
        dtp = ctypes.c_double()
        have = ctypes.c_int()
        _lib.check(self._lib.smc_get_history(self._h, prev.ctypes.data_as(ctypes.c_void_p),
                                             psi.ctypes.data_as(ctypes.c_void_p), _lib.SMC_HOST,
                                             ctypes.byref(dtp), ctypes.byref(have)))
        return dict(prev=prev, psi_prev=psi, dt_prev=float(dtp.value), have_prev=bool(have.value))

    def set_history(self, prev=None, psi_prev=None, dt_prev=0.0, have_prev=False):
        """Install a BDF2 history (as returned by :meth:`get_history`)."""
        if have_prev:
            a = np.ascontiguousarray(prev, dtype=np.complex128)
            b = np.ascontiguousarray(psi_prev, dtype=np.complex128)
            if a.shape != (self.Nk, self.Nz) or b.shape != (self.Nk, self.Nz):
                raise ValueError("history arrays must be (Nk, Nz) = (%d, %d)" % (self.Nk, self.Nz))
            _lib.check(self._lib.smc_set_history(self._h, a.ctypes.data_as(ctypes.c_void_p),
                                                 b.ctypes.data_as(ctypes.c_void_p), _lib.SMC_HOST,
                                                 float(dt_prev), 1))
        else:
            _lib.check(self._lib.smc_set_history(self._h, None, None, _lib.SMC_HOST, 0.0, 0))

    # ---------------------------------------------------------- physics
    def stokes(self, that):
        p, mem, keep = self._spec_in(that)
        dev = mem == _lib.SMC_DEVICE
        q1, psi = self._spec_out(dev)
        q2, om = self._spec_out(dev)
        _lib.check(self._lib.smc_stokes(self._h, p, mem, q1, q2))
        return psi, om

    def velocity(self, psi):
        p, mem, keep = self._spec_in(psi)
        dev = mem == _lib.SMC_DEVICE
        q1, ux = self._grid_out(self.Nx, dev)
        q2, uz = self._grid_out(self.Nx, dev)
        _lib.check(self._lib.smc_velocity(self._h, p, mem, q1, q2))
        return ux, uz

    def diagnostics(self, that):
        p, mem, keep = self._spec_in(that)
        d = _lib.SmcDiag()
        _lib.check(self._lib.smc_diagnostics(self._h, p, mem, ctypes.byref(d)))
        return {k: float(getattr(d, k)) for k, _ in _lib.SmcDiag._fields_}

    def dissipation_eta(self):
        """-> the viscosity the last Stokes solve consumed, which weights the
        (Di/Ra) Phi source: None on the isoviscous model (eta = 1), the bounded
        depth profile eta(z) (Nz,) on the eta_z model and on the eta_T model
        before its first solve, else the eta_T model's last (Nx, Nz) field
        (rbc_galerkin.py:375-383, convection_modes.py:215-222,
        coupled_model.py:499-507)."""
        buf = np.empty((self.Nx, self.Nz), dtype=np.float64)
        rows = ctypes.c_int(0)
        _lib.check(self._lib.smc_dissipation_eta(self._h, buf.ctypes.data_as(ctypes.c_void_p),
                                                 _lib.SMC_HOST, ctypes.byref(rows)))
        if rows.value == 0:
            return None
        return buf[0].copy() if rows.value == 1 else buf

    def dissipation_phi(self, psi):
        """-> Phi on the padded (2 Nx, Nz) grid for ``psi``, weighted with
        ``dissipation_eta()`` (rbc_galerkin.py:385-394)."""
        from .energy import phi_padded
        return phi_padded(self, psi, self.dissipation_eta())

    def mirror_error(self, that):
        """-> max |theta(x) - theta(Lx - x)| / max |theta| on the grid
        (rbc_galerkin.py:455-463)."""
        from .drivers import mirror_error
        return mirror_error(self, that)

    def run(self, that, tstop, dt=None, safety=0.5, dtmax=5e-3, cadence=200, verbose=True):
        """The simple march of rbc_galerkin.py:473-491: -> (state, diagnostics
        every ``cadence`` steps)."""
        from .drivers import run
        return run(self, that, tstop, dt=dt, safety=safety, dtmax=dtmax, cadence=cadence,
                   verbose=verbose)

    def project_mirror(self, that):
        p, mem, keep = self._spec_in(that)
        q, out = self._spec_out(mem == _lib.SMC_DEVICE)
        _lib.check(self._lib.smc_project_mirror(self._h, p, q, mem))
        return out

    # --------------------------------------------------------- transforms
    def _transform_spec(self, kind, cf, Ng):
        p, mem, keep = self._spec_in(cf)
        q, out = self._grid_out(Ng, mem == _lib.SMC_DEVICE)
        _lib.check(self._lib.smc_transform(self._h, kind, p, q, mem))
        return out

    def _transform_grid(self, kind, g, Ng):
        if self._is_device(g):
            import torch
            t = g.to(torch.float64).contiguous()
            p, mem, keep = ctypes.c_void_p(t.data_ptr()), _lib.SMC_DEVICE, t
        else:
            a = np.ascontiguousarray(np.asarray(g), dtype=np.float64)
            p, mem, keep = a.ctypes.data_as(ctypes.c_void_p), _lib.SMC_HOST, a
        if tuple(keep.shape) != (Ng, self.Nz):
            raise ValueError("grid must be (%d, %d)" % (Ng, self.Nz))
        q, out = self._spec_out(mem == _lib.SMC_DEVICE)
        _lib.check(self._lib.smc_transform(self._h, kind, p, q, mem))
        return out

    def grid(self, cf):
        """(Nk,Nz) coefficients -> (Nx,Nz) values (rbc_galerkin.py:322-325)."""
        return self._transform_spec(_lib.SMC_GRID, cf, self.Nx)

    def coeffs(self, g):
        """(Nx,Nz) values -> (Nk,Nz) coefficients (rbc_galerkin.py:327-330)."""
        return self._transform_grid(_lib.SMC_COEFFS, g, self.Nx)

    def _synth_pad(self, cf):
        return self._transform_spec(_lib.SMC_SYNTH_PAD, cf, self.Np)

    def _trunc_pad(self, g):
        return self._transform_grid(_lib.SMC_TRUNC_PAD, g, self.Np)

    def seed(self, amp=1e-3, m=1, n=1):
        """amp cos(m pi x) sin(n pi z) as coefficients (rbc_galerkin.py:494-497)."""
        X, Z = np.meshgrid(self.x, self.z, indexing="ij")
        return self.coeffs(amp * np.cos(m * np.pi * X) * np.sin(n * np.pi * Z))

    def vol_mean(self, g):
        return float(np.sum(self.wq * np.asarray(g).real.mean(axis=0)))

    # ----------------------------------------------------------- counters
    def counters(self):
        c = _lib.SmcCounters()
        _lib.check(self._lib.smc_counters_get(self._h, ctypes.byref(c)))
        return {k: getattr(c, k) for k, _ in _lib.COUNTER_FIELDS}

    def __getattr__(self, name):
        if name.startswith("n_") or name.startswith("last_") or name in (
                "max_T_excursion", "theta_last_iters", "theta_last_res"):
            h = self.__dict__.get("_h")
            if h:
                c = self.counters()
                if name in c:
                    return c[name]
        raise AttributeError(name)

    def describe(self):
        d = dict(mode=type(self).__name__, backend="gb300", form=self.form, Nx=self.Nx, Nz=self.Nz,
                 Ra=self.Ra, Lx=self.Lx, deta_T=self.deta_T,
                 internal_heating=self.internal_heating,
                 dissipation_number=self.dissipation_number,
                 compressibility=self.compressibility, tala_active=self.tala_active,
                 tala_a=self.tala_a)
        d.update(self.counters())
        return d


class ThetaSolverView:
    """The temperature solver's state under the names of the reference's
    ImplicitThetaSolver (core/implicit_theta.py:128-212, 496-521), read from
    the model's counters and configuration."""

    _COUNTERS = dict(last_iters="theta_last_iters", last_res="theta_last_res",
                     n_nonconv="n_theta_nonconv", n_be_fallback="n_be_fallback",
                     n_solves="n_theta_solves")

    def __init__(self, model):
        self._model = model

    def __getattr__(self, name):
        key = ThetaSolverView._COUNTERS.get(name)
        if key is None:
            raise AttributeError(name)
        return self._model.counters()[key]

    @property
    def scheme(self):
        return "bdf2"

    @property
    def rtol(self):
        return float(self._model._cfg.theta_rtol)

    @property
    def restart(self):
        return int(self._model._cfg.theta_restart)

    @property
    def maxiter(self):
        return int(self._model._cfg.theta_maxiter)

    @property
    def internal_heating(self):
        return self._model.internal_heating

    @property
    def dissipation_number(self):
        return self._model.dissipation_number


class RBC(GpuModel):
    """Isoviscous model: explicit advection + backward-Euler diffusion."""
    _MODEL = _lib.SMC_MODEL_CONST


class RBCImplicitTheta(GpuModel):
    """Frozen eta(z) Stokes + linearly-implicit BDF2 temperature step."""
    _MODEL = _lib.SMC_MODEL_ETA_Z

    @property
    def theta(self):
        """The temperature solver's state (ImplicitThetaSolver names)."""
        return ThetaSolverView(self)


class RBCCoupled(GpuModel):
    """eta(T(x,z,t)) coupled Stokes (lagged LU + defect / BFBT) + BDF2 theta."""
    _MODEL = _lib.SMC_MODEL_ETA_T

    @property
    def theta(self):
        """The temperature solver's state (ImplicitThetaSolver names)."""
        return ThetaSolverView(self)

    def eta_of(self, that):
        """-> the (Nx, Nz) viscosity of a state: padded law, window, x-truncation
        and positivity guard (models/coupled_model.py:401-496).  Updates the
        eta counters as the reference's eta_of does."""
        p, mem, keep = self._spec_in(that)
        q, out = self._grid_out(self.Nx, mem == _lib.SMC_DEVICE)
        _lib.check(self._lib.smc_eta_of(self._h, p, mem, q))
        return out
