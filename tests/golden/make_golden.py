"""Generate the golden fixtures under tests/golden/ from the SpecMC reference.

Run once, in a container where the reference package is importable:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py <reference checkout> [case ...]

(the first argument is required: the directory that holds the reference's
``specmc`` package; it may also be given as $SPECMC_REFERENCE with ``-`` in
its place)

(the optional case names restrict the run to those fixtures, e.g.
``arrhenius_pv_32x24``).

Every fixture is a small ``.npz`` written by the reference's own public API
(``specmc.api.build_model`` / ``march_adaptive`` / ``model.diagnostics``) or
by its own transform / operator objects, on seeded inputs built here.  Nothing
in the test suite imports the reference: the tests read only these files.

Fixtures (sizes chosen so the whole script runs in a few minutes):

* ``transforms_16x12.npz`` -- ``RBC.grid / coeffs / _synth_pad / _trunc_pad``
  and the basis matrices on a seeded random coefficient field.
* ``march_<case>.npz`` -- initial state, every step's dt and state, the final
  diagnostics and the model's counters for one adaptive march per case.
* ``pv_calibration.npz`` -- ``reference_state.calibrate_pv`` for both
  anchors (rows: anchor, V, deta_T, E, V, Ts, C, ln D; -1 = not given).
* ``energy_32x24.npz`` -- ``physics/heating.py`` / ``physics/dissipation.py``
  budgets and integrals on three states of the Arrhenius + H + Phi march.
* ``config_cases.json`` -- ``ConvectionConfig`` on 300 seeded configurations:
  outcome class, warning classes, ``canonical()``.
* ``ckpt/t_0.125000.npz`` -- a state written by ``specmc.io.checkpoint.save``.
* ``rheology.npz`` -- ``physics/viscosity.py``, ``physics/arrhenius.py`` and
  ``physics/eta_bounds.py`` on seeded sample points.
* ``physics_helpers.json`` -- closed forms and helpers of
  ``physics/heating.py`` and ``physics/dissipation.py``.
* ``drivers_32x24.npz`` -- ``RBC.run`` records and ``RBC.mirror_error``.
* ``initial_32x24.npz`` + ``aspect_synthetic.txt`` -- ``core/bench_ic.py``
  and ``physics/heating.py`` initial states (the ASPECT reader on a seeded
  synthetic file in that format).
* ``tala_ops_16x12.npz`` -- the TALA Stokes operators (``TalaStokes``,
  ``TalaFreeOperator``) and the TALA temperature operator, preconditioner and
  adiabatic source on one seeded state.
* ``coupled_ops_16x12.npz`` -- ``eta_of``, ``FreeSchurOperator.matvec``, the
  assembled Schur matrix and the BFBT preconditioner action for one seeded
  state (pins the coupled operator, including its partner half).
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def seeded_noise_theta(model, amp, mmax, nmax, seed, Lx, H=0.0):
    """Conductive profile (H) plus seeded mirror-symmetric noise, as coeffs.

    noise = sum_{m<=mmax, n<=nmax} a_mn cos(2 pi m x / Lx) sin(n pi z),
    a_mn ~ U(-1, 1), scaled so max|noise| = amp on the model grid.
    """
    rng = np.random.default_rng(seed)
    a = rng.uniform(-1.0, 1.0, size=(mmax, nmax))
    X, Z = np.meshgrid(model.x, model.z, indexing='ij')
    g = np.zeros_like(X)
    for m in range(1, mmax + 1):
        for n in range(1, nmax + 1):
            g += a[m - 1, n - 1] * np.cos(2.0 * np.pi * m * X / Lx) \
                * np.sin(n * np.pi * Z)
    g *= amp / np.abs(g).max()
    g += 0.5 * H * Z * (1.0 - Z)
    return model.coeffs(g)


COUNTER_KEYS = (
    'n_refresh', 'n_defect', 'n_defect_failed', 'n_defect_double_fail',
    'n_memo_hits', 'n_stokes', 'n_bfbt_solves', 'n_bfbt_iters',
    'n_bfbt_rescue', 'n_clip_eta', 'n_smooth_eta', 'n_clip_eta_proj',
    'n_steps')


def counters(m):
    out = {}
    for k in COUNTER_KEYS:
        if hasattr(m, k):
            out['ctr_' + k] = np.int64(getattr(m, k))
    th = getattr(m, 'theta', None)
    if th is not None:
        out['ctr_theta_n_nonconv'] = np.int64(th.n_nonconv)
        out['ctr_theta_n_be_fallback'] = np.int64(th.n_be_fallback)
        out['ctr_theta_last_iters'] = np.int64(th.last_iters)
    return out


def march_case(name, cfg_kw, steps, ic, S):
    api = S.api
    cfg = S.ConvectionConfig(**cfg_kw)
    m = api.build_model(cfg)
    if ic[0] == 'seed':
        th0 = m.seed(amp=ic[1], m=ic[2], n=ic[3])
    else:
        th0 = seeded_noise_theta(m, amp=ic[1], mmax=ic[2], nmax=ic[3],
                                 seed=ic[4], Lx=cfg.Lx,
                                 H=cfg.internal_heating)
    states, dts = [], []
    s = np.array(th0, copy=True)
    t = 0.0
    t0 = time.perf_counter()
    for _ in range(steps):
        dt = api.production_dt(m, s)
        s = m.step(s, dt)
        t += dt
        states.append(s.copy())
        dts.append(dt)
    el = time.perf_counter() - t0
    d = m.diagnostics(s)
    rec = dict(that0=th0, states=np.array(states), dts=np.array(dts),
               t=np.float64(t), wall_s=np.float64(el),
               **{'diag_' + k: np.float64(v) for k, v in d.items()},
               **counters(m))
    for k, v in cfg_kw.items():
        rec['cfg_' + k] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, 'march_%s.npz' % name), **rec)
    print('%-14s %3d steps  %.2f s  Nu_top=%.10f urms=%.10f'
          % (name, steps, el, d['Nu_top'], d['urms']), flush=True)


def long_march_case(name, cfg_kw, steps, ic, S, every=20):
    """A long adaptive march (the headline configurations at their own
    lengths): every step's dt, the diagnostics and the state every `every`
    steps and at the end, and the counters.  Written as ``long_<name>.npz``."""
    api = S.api
    cfg = S.ConvectionConfig(**cfg_kw)
    m = api.build_model(cfg)
    if ic[0] == 'seed':
        th0 = m.seed(amp=ic[1], m=ic[2], n=ic[3])
    else:
        th0 = seeded_noise_theta(m, amp=ic[1], mmax=ic[2], nmax=ic[3],
                                 seed=ic[4], Lx=cfg.Lx,
                                 H=cfg.internal_heating)
    keys = ('Nu_top', 'Nu_bot', 'Nu_energy', 'urms', 'umax', 'amp')
    dts, trace_steps, trace, trace_states, ts = [], [], [], [], []
    s = np.array(th0, copy=True)
    t = 0.0
    t0 = time.perf_counter()
    for i in range(steps):
        dt = api.production_dt(m, s)
        s = m.step(s, dt)
        t += dt
        dts.append(dt)
        if (i + 1) % every == 0 or i + 1 == steps:
            d = m.diagnostics(s)
            trace_steps.append(i + 1)
            ts.append(t)
            trace.append([d[k] for k in keys])
            trace_states.append(s.copy())
    el = time.perf_counter() - t0
    rec = dict(that0=th0, dts=np.array(dts), trace_steps=np.array(trace_steps),
               trace_t=np.array(ts), trace=np.array(trace),
               trace_keys=np.array(keys), trace_states=np.array(trace_states),
               state=s, t=np.float64(t), wall_s=np.float64(el), **counters(m))
    for k, v in cfg_kw.items():
        rec['cfg_' + k] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, 'long_%s.npz' % name), **rec)
    d = m.diagnostics(s)
    print('long %-14s %4d steps  %.1f s  t=%.6g Nu_top=%.10f urms=%.10f'
          % (name, steps, el, t, d['Nu_top'], d['urms']), flush=True)


def transforms_case(S):
    from specmc.core.rbc_galerkin import RBC
    rng = np.random.default_rng(7)
    m = RBC(Ra=1e4, Nx=16, Nz=12)
    cf = rng.standard_normal((m.Nk, m.Nz)) + 1j * rng.standard_normal((m.Nk, m.Nz))
    g = rng.standard_normal((m.Nx, m.Nz))
    gp = rng.standard_normal((m.Np, m.Nz))
    psi, om = m.stokes(cf)
    ux, uz = m.velocity(psi)
    np.savez_compressed(
        os.path.join(HERE, 'transforms_16x12.npz'),
        cf=cf, g=g, gp=gp, grid=m.grid(cf), coeffs=m.coeffs(g),
        synth_pad=m._synth_pad(cf), trunc_pad=m._trunc_pad(gp),
        V=m.V, Vi=m.Vi, D=m.D, z=m.z, x=m.x, kx=m.kx, wq=m.wq,
        psi=psi, om=om, ux=ux, uz=uz, step=m.step(cf, 1e-4),
        seed=m.seed(amp=3e-2, m=1, n=1))
    print('transforms_16x12 written', flush=True)


def coupled_ops_case(S):
    from specmc.models.coupled_model import RBCCoupled
    from specmc.stokes.lagged_stokes import FreeSchurOperator
    from specmc.stokes.stokes_coupled import CoupledStokes
    from specmc.stokes.bfbt import SpectralBFBTPrecond
    m = RBCCoupled(Nx=16, Nz=12, deta_T=1000.0, eta_drift_tol=0.1,
                   defect_tol=1e-8)
    th = seeded_noise_theta(m, amp=0.3, mmax=4, nmax=4, seed=11, Lx=m.Lx)
    eta = m.eta_of(th)
    rng = np.random.default_rng(3)
    n = m.Nk * m.Nz
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    op = CoupledStokes(m, eta)
    fop = FreeSchurOperator(m, eta, op_template=op)
    P = SpectralBFBTPrecond(m, eta, profile='harm')
    G = np.array([op.green(i) for i in range(m.Nk)])
    psi, om = m.stokes(th)
    np.savez_compressed(
        os.path.join(HERE, 'coupled_ops_16x12.npz'),
        that=th, eta=eta, v=v, Av=fop.matvec(v), A=op.assemble_schur(),
        b=op.rhs_schur(th), Pv=P.apply(v), G=G, eta_c=fop.eta_c,
        psi=psi, om=om)
    print('coupled_ops_16x12 written', flush=True)


def tala_ops_case(S):
    """The TALA operators (stokes/stokes_tala.py) on one seeded state of the
    eta_T model with Di = 0.7: eta, the L^(rho) Green functions, the assembled
    Schur matrix, the matrix-free action, the rho_bar^2 right-hand side, the
    unpacked (Psi, omega), and after one step the temperature operator, its
    rho_bar preconditioner and the adiabatic source."""
    from specmc.stokes.stokes_tala import TalaFreeOperator, TalaStokes
    api = S.api
    cfg = S.ConvectionConfig(Ra=1e4, Nx=16, Nz=12, viscosity_model='eta_T',
                             compressibility='tala', dissipation_number=0.7,
                             precond='legacy')
    m = api.build_model(cfg)
    rng = np.random.default_rng(3)
    th = m.seed(amp=0.2, m=1, n=1) + 0.05 * (rng.standard_normal((m.Nk, m.Nz))
                                            + 1j * rng.standard_normal((m.Nk, m.Nz)))
    eta = m.eta_of(th)
    op = TalaStokes(m, eta)
    fop = TalaFreeOperator(m, eta, op_template=op)
    v = rng.standard_normal(m.Nk * m.Nz) + 1j * rng.standard_normal(m.Nk * m.Nz)
    psi_v, om_v, _ = op.unpack_schur(v)
    th1 = m.step(th, 2e-5)
    tv = rng.standard_normal(m.Nk * m.Nz) + 1j * rng.standard_normal(m.Nk * m.Nz)
    rec = dict(that=th, eta=eta, v=v, Av=fop.matvec(v), A=op.assemble_schur(),
               b=op.rhs_schur(th), G=np.array([op.green(i) for i in range(m.Nk)]),
               psi_v=psi_v, om_v=om_v, rho_grid=m.rho_grid, rho_c=m.rho_c,
               rho2_c=m.rho2_c, tala_a=np.float64(m.tala_a), dt=np.float64(2e-5),
               that1=th1, tv=tv, theta_Av=m.theta.matvec(tv),
               theta_Pv=m.theta.precond(tv),
               adiabatic=m.theta._tala_adiabatic_source(m.project_mirror(th)))
    np.savez_compressed(os.path.join(HERE, 'tala_ops_16x12.npz'), **rec)
    print('tala_ops_16x12 written', flush=True)


def initial_conditions_case(S):
    """core/bench_ic.py and physics/heating.py initial states at 32x24: the
    conductive seed, the analytic boundary-layer state, the heated conductive
    profile, and an ASPECT ascii field read from a seeded synthetic file in
    that format (aspect_synthetic.txt; the benchmark's own file is not
    shipped) with the pchip and spline z-interpolants."""
    from specmc.core import bench_ic as B
    from specmc.core.rbc_galerkin import RBC
    from specmc.physics import heating as HEAT
    rng = np.random.default_rng(21)
    n = 16
    c = (np.arange(n) + 0.5) / n
    T = (1.0 - c)[:, None] + 0.05 * rng.uniform(-1.0, 1.0, (n, n)) * np.sin(np.pi * c)[:, None]
    path = os.path.join(HERE, 'aspect_synthetic.txt')
    with open(path, 'w') as f:
        f.write('# seeded synthetic temperature field in the ASPECT ascii-data layout\n')
        f.write('# POINTS: %d %d\n' % (n, n))
        for j in range(n):
            for i in range(n):
                f.write('%.10f %.10f %.15e\n' % (c[i], c[j], T[j, i]))
    m = RBC(Ra=1e4, Nx=32, Nz=24)
    np.savez_compressed(
        os.path.join(HERE, 'initial_32x24.npz'),
        conductive=B.conductive_theta(m, amp=3e-2, m=2, n=1),
        analytic_bl=B.analytic_bl_theta(m),
        heated=HEAT.conductive_theta(m.z, 1.5),
        aspect_pchip=B.aspect_theta(m, path=path, zinterp='pchip'),
        aspect_spline=B.aspect_theta(m, path=path, zinterp='spline'))
    print('initial_32x24 written', flush=True)


def drivers_case(S):
    """RBC.run (core/rbc_galerkin.py:473-491) on the isoviscous 32x24 model,
    30 CFL steps with diagnostics every 10, and RBC.mirror_error of a
    mirror-symmetric and of a seeded non-symmetric state."""
    from specmc.core.rbc_galerkin import RBC
    m = RBC(Ra=1e4, Nx=32, Nz=24)
    th0 = m.seed(amp=3e-2, m=1, n=1)
    s, hist = m.run(th0, tstop=30 * 4e-5 * 0.999, safety=0.5, dtmax=4e-5, cadence=10,
                    verbose=False)
    keys = sorted(hist[0])
    rng = np.random.default_rng(8)
    odd = rng.standard_normal((m.Nk, m.Nz)) + 1j * rng.standard_normal((m.Nk, m.Nz))
    np.savez_compressed(os.path.join(HERE, 'drivers_32x24.npz'), that0=th0, final=s,
                        keys=np.array(keys), hist=np.array([[h[k] for k in keys] for h in hist]),
                        odd=odd, mirror_sym=np.float64(m.mirror_error(s)),
                        mirror_odd=np.float64(m.mirror_error(odd)), n_steps=np.int64(m.n_steps))
    print('drivers_32x24 written', flush=True)


def physics_helpers_case(S):
    """The closed forms and helpers of physics/heating.py and
    physics/dissipation.py on sample arguments, and phi_z_tail /
    source_coeffs on the third state of the energy fixture's march."""
    import json
    from specmc.physics import heating as HEAT, dissipation as DISS
    z = np.linspace(0.0, 1.0, 7)
    out = {}
    for H in (0.0, 1.5, 2.0, 4.0, -1.0):
        out['H=%g' % H] = dict(
            conductive_theta=HEAT.conductive_theta(z, H).tolist(),
            conductive_T=HEAT.conductive_T(z, H).tolist(),
            mean_T=HEAT.mean_T_conductive(H), nu_bot=HEAT.nu_bot_conductive(H),
            nu_top=HEAT.nu_top_conductive(H), T_max=list(HEAT.T_max_conductive(H)),
            nu_energy=HEAT.nu_energy_steady(0.3, H), nu_bot_energy=HEAT.nu_bot_energy_steady(0.3, H),
            nu_top_steady=DISS.nu_top_steady(0.3, H, 0.05),
            nu_bot_steady=DISS.nu_bot_steady(0.3, H, 0.05),
            source_integral=HEAT.source_integral(H),
            source_00=HEAT.source_coeffs(3, 4, H)[0, 0].real)
    out['single_mode'] = [DISS.single_mode_theta_integral(1e4, np.pi, np.pi, 1.0),
                          DISS.single_mode_theta_integral(3e5, 2 * np.pi, np.pi, 0.2),
                          DISS.single_mode_psi_integral(np.pi, 2 * np.pi, -3.0)]
    rng = np.random.default_rng(2)
    prof = rng.uniform(0.5, 2.0, 5)
    cases = [None, np.ones((4, 5)), prof, np.tile(prof, (4, 1)), rng.uniform(0.5, 2.0, (4, 5))]
    out['eta_class'] = [DISS.eta_class(c) for c in cases]
    out['j9_2_bound'] = [DISS.j9_2_bound(c, t, p) for c in ('const', 'eta_z', 'eta_xz', 'other')
                         for t, p in ((0.0, 0.0), (1e-8, 0.0), (0.0, 1e-3))]
    g = np.load(os.path.join(HERE, 'energy_32x24.npz'))
    api = S.api
    cfg = S.ConvectionConfig(Ra=1e4, Nx=32, Nz=24, viscosity_model='arrhenius', deta_T=1e3,
                             arrhenius_Ts=1.0, eta_min=1e-3, eta_max=1.0,
                             dissipation_number=0.5, internal_heating=1.0)
    m = api.build_model(cfg)
    out['phi_z_tail'] = DISS.phi_z_tail(m, g['psi'], g['eta'])
    sc = DISS.source_coeffs(m, g['psi'], g['eta'], Di=0.5)
    out['source_coeffs_norm'] = float(np.linalg.norm(sc))
    out['source_coeffs_integral'] = DISS.source_integral(m, sc)
    from specmc.core import cfl_policy as CFL
    from specmc.core.rbc_galerkin import RBC
    r = RBC(Ra=1e4, Nx=32, Nz=24)
    th = r.seed(amp=3e-2, m=1, n=1)
    out['cfl'] = [CFL.cfl_dt(r, th, safety=sf, dtmax=dm, clamp=cl)
                  for sf in (0.4, 40.0, 500.0, -1.0) for dm in (4e-5, 1.0) for cl in (True, False)
                  if not (sf < 0 and not cl)]
    out['clamp_safety'] = [CFL.clamp_safety(v) for v in (-3.0, 0.5, 40.0, 100.0)]
    with open(os.path.join(HERE, 'physics_helpers.json'), 'w') as f:
        json.dump(out, f, indent=0, sort_keys=True)
    print('physics_helpers written', flush=True)


def rheology_case(S):
    """physics/viscosity.py, physics/arrhenius.py and physics/eta_bounds.py on
    seeded sample points."""
    from specmc.physics import arrhenius as AR, eta_bounds as EB, viscosity as VI
    rng = np.random.default_rng(13)
    T = np.concatenate(([0.0, 1.0, 2.0], rng.uniform(0.0, 2.0, 29)))
    z = rng.uniform(0.0, 1.0, T.size)
    eta = np.exp(rng.uniform(np.log(1e-5), np.log(1e5), 64))
    eta[:4] = [1e-3, 1e-3 * (1.0 - 1e-13), 1e3 * (1.0 + 1e-13), 1e3]
    E, V, Ts = AR.arrhenius_E(1e3, 0.3), 0.7, 0.3
    rec = dict(
        T=T, z=z, eta=eta,
        eta_exp_T=VI.eta_exp_T(T, 1e3),
        eta_background=VI.eta_conductive_background(z, 100.0),
        eta_law_iso=VI.eta_from_law('isoviscous', 100.0, z),
        eta_law_exp=VI.eta_from_law('exp_T_depth', 100.0, z),
        arr_scalars=np.array([AR.arrhenius_E(1e3, 0.3), AR.arrhenius_C(1e3, 0.3),
                              AR.cold_end_slope(1e3, 0.3), AR.slope_amplification(0.3),
                              AR.infer_deta_T(5.0, 0.3), AR.infer_Ts(5.0, 1e3),
                              AR.hot_end_contrast_V(T, z, E, V, Ts)]),
        arr_exponent=AR.arrhenius_exponent(T, 1e3, 0.3),
        arr_eta=AR.eta_arrhenius_T(T, 1e3, 0.3),
        arr_exponent_V=AR.arrhenius_exponent_V(T, z, E, V, Ts),
        arr_eta_V=AR.eta_arrhenius_V(T, z, E, V, Ts),
        windows=np.array([*EB.reachable_window(1e3), *EB.reachable_window_arrhenius(1e3, 1.0),
                          *EB.reachable_window_arrhenius(1e3, 0.05),
                          *EB.reachable_window_pv(E, V, Ts), *EB.effective_bounds(1e-3, 1e3)]),
        n_clipped=np.int64(EB.n_clipped(eta, 1e-3, 1e3)),
        clip=EB.clip_eta(eta, 1e-3, 1e3)[0], clip_n=np.int64(EB.clip_eta(eta, 1e-3, 1e3)[1]),
        smoothstep=EB.smoothstep5(np.linspace(-0.5, 1.5, 21)),
        n_band=np.int64(EB.n_in_transition(eta, 1e-3, 1e3, 1.5)),
        smooth=EB.smooth_clip_eta(eta, 1e-3, 1e3, 1.5)[0],
        smooth_n=np.int64(EB.smooth_clip_eta(eta, 1e-3, 1e3, 1.5)[1]))
    np.savez_compressed(os.path.join(HERE, 'rheology.npz'), **rec)
    print('rheology written', flush=True)


def pv_calibration_case(S):
    """reference_state.calibrate_pv for both anchors and a few V-tilde /
    contrast values (the pV(L) law's Ts, E-tilde, V-tilde, C, ln D)."""
    from specmc.physics.reference_state import calibrate_pv
    rows = []
    for anchor, V, D in (("Ea", None, None), ("Ea", 2.0, None), ("D", 2.0, 1e3),
                         ("D", 0.5, 1e5), ("D", 22.5, 10.0)):
        r = calibrate_pv(anchor=anchor, V=V, deta_T=D)
        rows.append([0 if anchor == "Ea" else 1, -1.0 if V is None else V,
                     -1.0 if D is None else D, r["E"], r["V"], r["Ts"], r["C"], r["ln_D"]])
    np.savez_compressed(os.path.join(HERE, 'pv_calibration.npz'), rows=np.array(rows))
    print('pv_calibration written', flush=True)


def energy_case(S):
    """physics/heating.py and physics/dissipation.py diagnostics on three
    states of the Arrhenius + H + Phi march: the BDF2 budgets, <Phi>,
    Ra <theta u_z>, the flux profile and the boundary fluxes."""
    from specmc.physics import heating as HEAT, dissipation as DISS
    api = S.api
    cfg = S.ConvectionConfig(Ra=1e4, Nx=32, Nz=24, viscosity_model='arrhenius', deta_T=1e3,
                             arrhenius_Ts=1.0, eta_min=1e-3, eta_max=1.0,
                             dissipation_number=0.5, internal_heating=1.0)
    m = api.build_model(cfg)
    s0 = seeded_noise_theta(m, amp=1e-2, mmax=8, nmax=8, seed=99, Lx=cfg.Lx, H=1.0)
    states = [s0]
    for _ in range(3):
        states.append(m.step(states[-1], api.production_dt(m, states[-1])))
    s1, s2, s3 = states[1], states[2], states[3]
    psi, _ = m.stokes(s3)
    eta = m.eta_of(s3)
    a0, b0, b1 = 3.5e4, 4.6e4, 1.1e4
    hb = HEAT.balance(m, s3, s2, s1, a0, b0, b1, H=1.0)
    db = DISS.balance(m, s3, s2, s1, a0, b0, b1, H=1.0, Di=0.5, psi=psi, eta=eta)
    z, q = HEAT.flux_profile(m, s3, H=1.0)
    rec = dict(s1=s1, s2=s2, s3=s3, psi=psi, eta=eta, abc=np.array([a0, b0, b1]),
               phi_int=np.float64(DISS.phi_integral(m, psi, eta)),
               phi_int_noeta=np.float64(DISS.phi_integral(m, psi)),
               pi_theta=np.float64(DISS.pi_theta(m, psi, s3)),
               pi_theta_plain=np.float64(DISS.pi_theta(m, psi, s3, dealias=False)),
               phi_coeffs=DISS.phi_coeffs(m, psi, eta), q=q,
               **{'hb_' + k: np.float64(v) for k, v in hb.items()},
               **{'db_' + k: np.float64(v) for k, v in db.items()})
    np.savez_compressed(os.path.join(HERE, 'energy_32x24.npz'), **rec)
    print('energy_32x24 written', flush=True)


CONFIG_MENU = dict(
    viscosity_model=['eta_T', 'const', 'eta_z', 'arrhenius', 'constant', 'isoviscous', 'etaz',
                     'nope', 'eta_Tz', 'ETA_T'],
    deta_T=[1000.0, 1.0, 0.5, -1.0, 1e5],
    eta_z_coeff=[0.0, 1.0], depth_dependence=[0.0, 0.5],
    arrhenius_E=[0.0, 1.0, 7.536], arrhenius_V=[0.0, 0.5, -1.0, 2.0],
    reference_anchor=['D', 'Ea', 'X'], arrhenius_Ts=[0.0, 1.0, 0.091, -0.5],
    eta_min=[1e-3, 1.0, 0.0, -1.0, 1e-6], eta_max=[1e3, 1.0, 0.5, 1e6],
    eta_smooth=[0.0, 0.5, 2.0, -0.1], precond=['legacy', 'bfbt', 'ilu', 'BFBT'],
    internal_heating=[0.0, 1.5, -1.0], dissipation_number=[0.0, 0.5, -0.5],
    compressibility=['boussinesq', 'tala', 'ala', 'x'], Ra=[1e4, 0.0, -1.0, 1e7],
    Nx=[64, 3, 63, 32], Nz=[96, 3, 24], Lx=[2.0, 4.0, 0.0], lag=[16, 0, 1], K=[3, 0, 9, 8],
    defect_tol=[1e-8, 0.0, -1.0], max_K=[8, 0, 3], symmetrize=[True, False])


def config_case(S):
    """ConvectionConfig on 300 seeded configurations (1 to 3 fields moved from
    their defaults to edge values): the outcome class (ok or the exception),
    the warning classes and, when valid, canonical()."""
    import json
    import warnings
    rng = np.random.default_rng(5)
    names = sorted(CONFIG_MENU)
    out = []
    for _ in range(300):
        kw = {}
        for name in rng.choice(names, size=int(rng.integers(1, 4)), replace=False):
            vals = CONFIG_MENU[str(name)]
            v = vals[int(rng.integers(len(vals)))]
            kw[str(name)] = v.item() if hasattr(v, 'item') else v
        rec = dict(kw=kw)
        with warnings.catch_warnings(record=True) as w:
            warnings.simplefilter('always')
            try:
                c = S.ConvectionConfig(**kw)
                rec['outcome'] = 'ok'
                rec['canonical'] = c.canonical()
                try:
                    sp = S.api.model_spec(c)
                    rec['spec'] = dict(model=sp['model'], builder=sp['builder'],
                                       kwargs={k: (None if v is None else v)
                                               for k, v in sp['kwargs'].items()})
                    rec['describe'] = json.loads(json.dumps(S.api.describe(c), default=str))
                except Exception as ex:                 # noqa: BLE001
                    rec['spec'] = type(ex).__name__
            except Exception as ex:                     # noqa: BLE001 -- the class is the record
                rec['outcome'] = type(ex).__name__
        rec['warnings'] = sorted({x.category.__name__ for x in w})
        out.append(rec)
    with open(os.path.join(HERE, 'config_cases.json'), 'w') as f:
        json.dump(out, f, indent=0, sort_keys=True)
    print('config_cases written', flush=True)


def checkpoint_case(S):
    """A checkpoint written by specmc.io.checkpoint.save (the reference's own
    writer), under tests/golden/ckpt/."""
    from specmc.io import checkpoint as CK
    that = (np.arange(12.0) + 1j * np.arange(12.0)[::-1]).reshape(3, 4)
    d = os.path.join(HERE, 'ckpt')
    for f in os.listdir(d) if os.path.isdir(d) else ():
        os.remove(os.path.join(d, f))
    p = CK.save(d, that, 0.125, n=7, fac=40.0)
    print('checkpoint written:', os.path.basename(p), flush=True)


def main(ref_root, only=()):
    sys.path.insert(0, ref_root)
    import specmc.api as api
    from specmc.config import ConvectionConfig

    class S:
        pass
    S.api = api
    S.ConvectionConfig = ConvectionConfig
    def mc(name, *a):                    # the selected march cases only
        if not only or name in only:
            march_case(name, *a)

    if not only:
        transforms_case(S)
        coupled_ops_case(S)
    if not only or 'pv_calibration' in only:
        pv_calibration_case(S)
    if not only or 'energy_32x24' in only:
        energy_case(S)
    if not only or 'config_cases' in only:
        config_case(S)
    if not only or 'checkpoint' in only:
        checkpoint_case(S)
    if not only or 'tala_ops' in only:
        tala_ops_case(S)
    if not only or 'initial' in only:
        initial_conditions_case(S)
    if not only or 'drivers' in only:
        drivers_case(S)
    if not only or 'physics_helpers' in only:
        physics_helpers_case(S)
    if not only or 'rheology' in only:
        rheology_case(S)
    base = dict(Ra=1e4, Nx=32, Nz=24)
    # configuration 1 of the headline table: isoviscous, march to t = 1e-3
    mc('const_32x24', dict(base, viscosity_model='const'), 25,
               ('seed', 3e-2, 1, 1), S)
    mc('etaz_32x24', dict(base, viscosity_model='eta_z',
                                  deta_T=100.0), 20, ('seed', 3e-2, 1, 1), S)
    mc('etaT_32x24', dict(base, viscosity_model='eta_T'), 25,
               ('seed', 3e-2, 1, 1), S)
    mc('etaT_bfbt_32x24', dict(base, viscosity_model='eta_T',
                                       precond='bfbt'), 12,
               ('seed', 3e-2, 1, 1), S)
    # internally heated 2:1 box (Lx = 4 is the mirror-doubled carrier)
    mc('heated_2to1_32x24',
               dict(base, viscosity_model='eta_T', Lx=4.0, Ra=1.25e4,
                    internal_heating=1.5), 12,
               ('noise', 1e-2, 8, 8, 1234), S)
    # Arrhenius + window + dissipation + heating (the large-run physics)
    mc('arrhenius_32x24',
               dict(base, viscosity_model='arrhenius', deta_T=1e3,
                    arrhenius_Ts=1.0, eta_min=1e-3, eta_max=1.0,
                    dissipation_number=0.5, internal_heating=1.0),
               12, ('noise', 1e-2, 8, 8, 99), S)
    # smooth eta window that is active on this state
    mc('smooth_32x24',
               dict(base, viscosity_model='eta_T', eta_min=3e-3, eta_max=1.0,
                    eta_smooth=0.5), 10, ('seed', 3e-2, 1, 1), S)
    # the pressure-dependent Arrhenius law (pV(L), arrhenius_V > 0) with the
    # contrast anchor 'D' (E-tilde from deta_T), default viscosity window
    mc('arrhenius_pv_32x24',
               dict(base, viscosity_model='arrhenius', deta_T=1e3,
                    arrhenius_V=0.5, reference_anchor='D'),
               6, ('noise', 1e-2, 8, 8, 42), S)
    # the TALA operator route (compressibility='tala', Di = 0.25): the
    # velocity division on every route, the rho_bar-weighted temperature
    # equation on eta_z / eta_T, the TALA Schur operator on the legacy route
    tala = dict(base, compressibility='tala', dissipation_number=0.25)
    mc('tala_const_32x24', dict(tala, viscosity_model='const'), 8,
       ('seed', 3e-2, 1, 1), S)
    mc('tala_etaz_32x24', dict(tala, viscosity_model='eta_z', deta_T=100.0), 8,
       ('seed', 3e-2, 1, 1), S)
    mc('tala_etaT_32x24', dict(tala, viscosity_model='eta_T', precond='legacy'), 8,
       ('seed', 3e-2, 1, 1), S)
    mc('tala_arrhenius_32x24',
       dict(tala, viscosity_model='arrhenius', precond='legacy', deta_T=1e3,
            arrhenius_Ts=1.0, eta_min=1e-3, eta_max=1.0, internal_heating=1.0),
       6, ('noise', 1e-2, 8, 8, 99), S)
    # configuration 2 grid, a few steps (the oracle of the bench workload)
    mc('etaT_64x96', dict(Ra=1e4, Nx=64, Nz=96,
                                  viscosity_model='eta_T'), 6,
               ('seed', 3e-2, 1, 1), S)
    # the headline configurations at their own lengths (long_<name>.npz):
    # configuration 2, 200 adaptive steps on the default (legacy) route
    if not only or 'long_etaT_64x96' in only:
        long_march_case('etaT_64x96', dict(Ra=1e4, Nx=64, Nz=96, viscosity_model='eta_T',
                                           deta_T=1000.0), 200, ('seed', 3e-2, 1, 1), S)
    # configuration 3 (internally heated 2:1 box, Lx = 4 the mirror-doubled
    # carrier, seeded noise 1e-2 in m, n <= 8): its first 60 steps
    if not only or 'long_heated_2to1_64x96' in only:
        long_march_case('heated_2to1_64x96',
                        dict(Ra=1.25e4, Nx=64, Nz=96, viscosity_model='eta_T', deta_T=1000.0,
                             Lx=4.0, internal_heating=1.5), 60,
                        ('noise', 1e-2, 8, 8, 2025), S, every=10)


if __name__ == '__main__':
    if len(sys.argv) < 2:
        sys.exit('usage: make_golden.py <reference checkout | -> [case ...]')
    root = sys.argv[1]
    if root == '-':
        root = os.environ.get('SPECMC_REFERENCE', '')
    if not os.path.isdir(os.path.join(root, 'specmc')):
        sys.exit('no specmc package under %r' % root)
    main(root, tuple(sys.argv[2:]))
