/*
 * specmc_gb300 -- C ABI of the GB300 time step of SpecMC.
 *
 * The reference (SpecMC) is a pure-Python package with no FFI; its public
 * surface for this path is `ConvectionConfig` + `specmc.api.build_model /
 * march / march_adaptive / production_dt / describe` and the duck-typed model
 * object those functions drive (`step`, `cfl_dt`, `diagnostics`, `stokes`,
 * `grid`, `coeffs`, counters).  Each entry point below replaces one of those
 * calls; the comment names the reference function (file:line, paths inside
 * the reference repository) whose behaviour it reproduces.
 *
 * Conventions
 *   - Spectral state `that`: (Nk, Nz) complex128, row-major, interleaved
 *     (re, im) doubles, Nk = Nx/2 + 1.  Row k is the rfft mode kx = 2 pi k/Lx,
 *     column n the Chebyshev coefficient of T_n(2z - 1).
 *   - Grid fields: (Ng, Nz) float64 row-major, x node i, ascending CGL node j.
 *   - `mem` selects where a caller pointer lives: SMC_HOST (pageable or
 *     pinned host memory; copies happen inside the call) or SMC_DEVICE
 *     (device memory of the handle's GPU; no copy).
 *   - Return value: 0 success; < 0 hard error (the message is available from
 *     smc_last_error()).  Soft numerical trouble is never an error: it is
 *     counted in smc_counters, as the reference counts it.
 *   - A handle owns its device buffers and one CUDA stream; it is not
 *     re-entrant.  Different handles may be used from different threads.
 *   - No call reads or writes the caller's input buffers after it returns.
 */
#ifndef SPECMC_GB300_H
#define SPECMC_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define SMC_ABI_VERSION 3

enum smc_model { SMC_MODEL_CONST = 0, SMC_MODEL_ETA_Z = 1, SMC_MODEL_ETA_T = 2 };
enum smc_precond { SMC_PRECOND_LEGACY = 0, SMC_PRECOND_BFBT = 1 };
enum smc_precision { SMC_FP64 = 0, SMC_MIXED = 1 };
/* ConvectionConfig.compressibility (specmc/config.py:159-179): the
 * Boussinesq equations, or the truncated anelastic liquid approximation with
 * the reference density rho_bar = exp((1 - z) Di) of the run's
 * dissipation_number (core/rbc_galerkin.py:288-312) */
enum smc_compressibility { SMC_BOUSSINESQ = 0, SMC_TALA = 1 };
enum smc_mem { SMC_HOST = 0, SMC_DEVICE = 1 };
enum smc_transform {
  SMC_GRID = 0,       /* (Nk,Nz) coeffs -> (Nx,Nz) values   rbc_galerkin.py:322 */
  SMC_COEFFS = 1,     /* (Nx,Nz) values -> (Nk,Nz) coeffs   rbc_galerkin.py:327 */
  SMC_SYNTH_PAD = 2,  /* (Nk,Nz) coeffs -> (2Nx,Nz) values  rbc_galerkin.py:332 */
  SMC_TRUNC_PAD = 3   /* (2Nx,Nz) values -> (Nk,Nz) x-modes rbc_galerkin.py:338 */
};

/* One scenario, already translated from ConvectionConfig by the recipe
 * modules (specmc/models/{const,eta_z,eta_T}.py kwargs()).  Zero-initialise
 * and call smc_config_defaults() before filling it. */
typedef struct smc_config {
  int abi_version;          /* SMC_ABI_VERSION */
  int model;                /* enum smc_model (arrhenius = ETA_T with arrhenius_Ts > 0) */
  int Nx, Nz;
  double Ra, Lx, deta_T;
  double internal_heating;  /* H   */
  double dissipation_number;/* Di  */
  double eta_min, eta_max, eta_smooth;
  double arrhenius_Ts;      /* 0 = exponential law */
  int precond;              /* enum smc_precond */
  int symmetrize;
  int lag, K, max_K;
  double defect_tol;        /* <= 0 selects the fixed-K route */
  double eta_drift_tol;
  double stokes_rtol, theta_rtol;
  int theta_maxiter, theta_restart;
  int stokes_restart, stokes_maxiter;
  int precision;            /* enum smc_precision */
  int device;               /* CUDA ordinal */
  /* pressure-dependent Arrhenius law pV(L) (physics/arrhenius.py:283-327),
   * active when arrhenius_V > 0 (model ETA_T):
   *   ln eta = -E T / (Ts (T + Ts)) + V (1 - z) / (T + Ts),  Ts = arrhenius_Ts,
   * with E = E-tilde and V = V-tilde from the calibration
   * (physics/reference_state.py:277-364, done by the caller) */
  double arrhenius_E;
  double arrhenius_V;
  /* enum smc_compressibility.  SMC_TALA: u = curl(Psi) / rho_bar on every
   * model (rbc_galerkin.py:355-372); the rho_bar-weighted temperature
   * equation with the adiabatic source on ETA_Z / ETA_T
   * (implicit_theta.py:159-178, :332-493); the TALA Schur operator
   * (stokes/stokes_tala.py) on the legacy route of ETA_T.  SMC_TALA needs
   * precision SMC_FP64 and, on ETA_T, precond SMC_PRECOND_LEGACY (the
   * reference has no TALA form of the BFBT preconditioner, config.py:462-470). */
  int compressibility;
} smc_config;

typedef struct smc_handle smc_handle;

typedef struct smc_diag {   /* RBC.diagnostics, rbc_galerkin.py:439-453 */
  double Nu_top, Nu_bot, Nu_energy, urms, umax, amp;
} smc_diag;

typedef struct smc_counters {
  long long n_steps, n_stokes, n_memo_hits;
  long long n_refresh, n_defect, n_defect_failed, n_defect_double_fail;
  long long n_bfbt_solves, n_bfbt_iters, n_bfbt_rescue, n_bfbt_rescue_direct,
            n_bfbt_rescue_weak;
  long long n_clip_T, n_T_out_of_range, n_clip_eta, n_smooth_eta,
            n_clip_eta_proj, n_smooth_eta_proj;
  long long n_theta_nonconv, n_be_fallback, n_theta_solves, n_theta_iters;
  long long theta_last_iters, last_K;
  double max_T_excursion, last_corr, theta_last_res, last_bfbt_true_res,
         sym_removed;
  long long n_kernel_launches;       /* kernels this handle has launched */
} smc_counters;

typedef struct smc_march_info {     /* api.march_adaptive return dict */
  long long steps;
  double t, dt;
} smc_march_info;

/* Fill `cfg` with the production defaults (specmc/_numerics.py:67-148,
 * specmc/config.py:240-423). */
void smc_config_defaults(smc_config* cfg);

/* Build a model: api.build_model (specmc/api.py:102-110) -> RBC /
 * RBCImplicitTheta / RBCCoupled constructors (rbc_galerkin.py:258-315,
 * implicit_theta.py:557-599, coupled_model.py:128-330). */
int smc_create(const smc_config* cfg, smc_handle** out);
int smc_destroy(smc_handle* h);

/* model.step(that, dt) -> new state (rbc_galerkin.py:426, implicit_theta.py:608,
 * via the coupled model's memoised Stokes solve coupled_model.py:725). */
int smc_step(smc_handle* h, const double* that_in, double* that_out, int mem, double dt);

/* model.cfl_dt(that, safety, dtmax, dtmin) (rbc_galerkin.py:465-471). */
int smc_cfl_dt(smc_handle* h, const double* that_in, int mem, double safety,
               double dtmax, double dtmin, double* dt_out);

/* api.production_dt (api.py:126-133) = cfl_policy.cfl_dt (cfl_policy.py:64-73). */
int smc_production_dt(smc_handle* h, const double* that_in, int mem,
                      double safety, double dtmax, double* dt_out);

/* api.march_adaptive (api.py:169-190): CFL-limited march to tstop, the state
 * staying on the device between steps.  max_steps <= 0 means unbounded. */
int smc_march_adaptive(smc_handle* h, const double* that_in, double* that_out,
                       int mem, double tstop, double safety, double dtmax,
                       long long max_steps, smc_march_info* info);

/* api.march (api.py:147-166): fixed-dt march of nsteps. */
int smc_march(smc_handle* h, const double* that_in, double* that_out, int mem,
              double dt, long long nsteps);

/* Device-resident march (the state the C-ABI keeps between calls, as the
 * reference's march_adaptive keeps `s` between steps, api.py:179-189):
 * set_state uploads a state and restarts the march clock t = 0; advance runs
 * CFL-limited steps (production_dt + step) until t >= tstop or max_steps
 * (<= 0: unbounded); get_state downloads the current state.
 * Inside a march a step waits on the device twice (the Stokes-memo test, and
 * the CFL reduction that also carries the solve's result and the next memo
 * test); the result of the last temperature solve of smc_advance is read by
 * the next call's first wait, or by any other entry point of the handle before
 * it does anything else -- an error of that solve surfaces there. */
int smc_set_state(smc_handle* h, const double* that, int mem);
int smc_get_state(smc_handle* h, double* that_out, int mem);
int smc_advance(smc_handle* h, double tstop, long long max_steps, double safety,
                double dtmax, smc_march_info* info);

/* Kernel-region timing with CUDA events on the handle's stream (no
 * reference counterpart; the reference keeps wall-clock accumulators
 * t_stokes/t_refresh, coupled_model.py:329-330).  smc_profile(h, 1) resets
 * and enables every region, smc_profile(h, 2) only the Krylov engine regions
 * ("engine_stokes", "engine_theta": two events per solve, so a timed march
 * is not perturbed), smc_profile(h, 0) disables; smc_profile_get returns slot
 * `slot` (name NULL past the last):
 * total ms, launches, and the algorithmic work counted for those launches
 * (flops, or bytes when *work_is_bytes). */
int smc_profile(smc_handle* h, int enable);
int smc_profile_get(smc_handle* h, int slot, const char** name, double* ms,
                    long long* launches, double* work, int* work_is_bytes);

/* model.diagnostics(that) (rbc_galerkin.py:439-453). */
int smc_diagnostics(smc_handle* h, const double* that_in, int mem, smc_diag* out);

/* model.stokes(that) -> (psi, omega) coefficients (rbc_galerkin.py:342,
 * convection_modes.py:224, coupled_model.py:725). */
int smc_stokes(smc_handle* h, const double* that_in, int mem, double* psi_out,
               double* om_out);

/* model.velocity(psi) -> (ux, uz) on the (Nx,Nz) grid (rbc_galerkin.py:355). */
int smc_velocity(smc_handle* h, const double* psi_in, int mem, double* ux_out,
                 double* uz_out);

/* RBCVariableViscosity.project_mirror (convection_modes.py:134-153). */
int smc_project_mirror(smc_handle* h, const double* that_in, double* that_out, int mem);

/* The four transforms of the model (see enum smc_transform). */
int smc_transform(smc_handle* h, int kind, const double* in, double* out, int mem);

/* RBCCoupled.eta_of (coupled_model.py:401-496): the (Nx,Nz) viscosity the
 * coupled Stokes operator consumes for `that` (updates the eta counters). */
int smc_eta_of(smc_handle* h, const double* that_in, int mem, double* eta_out);

/* The viscosity the last Stokes solve consumed, the field the (Di/Ra) Phi
 * source is weighted with (dissipation_eta: rbc_galerkin.py:375-383,
 * convection_modes.py:215-222, coupled_model.py:499-507).  `eta_out` holds
 * Nx*Nz doubles; *rows_out = 0 (const model, eta = 1: nothing written), 1
 * (the bounded depth profile eta(z): Nz values; also the eta_T model before
 * its first Stokes solve) or Nx (the (Nx,Nz) field of the eta_T model's last
 * coupled solve). */
int smc_dissipation_eta(smc_handle* h, double* eta_out, int mem, int* rows_out);

/* FreeSchurOperator.matvec (stokes/lagged_stokes.py:202-220) at the viscosity
 * `eta` (Nx,Nz): out = A(eta) v, v and out (Nk,Nz) complex. */
int smc_schur_matvec(smc_handle* h, const double* eta, const double* v,
                     double* out, int mem);

/* Implementation switches with no reference counterpart (the reference has
 * one evaluation of each operator).  "dense_mult_eta" (0/1): evaluate
 * mult_eta with the dense per-shift Chebyshev product blocks
 * (stokes/lagged_stokes.py:162-193 term by term) instead of the default
 * pseudo-spectral form of the same linear map; used to cross-check them.
 * "schur_matvec_variant" (0/1/2, SMC_MIXED handles): which operator
 * smc_schur_matvec applies -- 0 the plain one, 1 the fused FP64 operator of
 * the fast form, 2 its FP32 inner-iteration operator.
 * "inner_fp32" (0/1, SMC_MIXED handles, default 1): run the fast form's
 * Krylov solves as FP32-operator inner FGMRES inside an FP64 refinement loop
 * (1) or as plain FP64 FGMRES on the fused operators (0).
 * "krylov_engine" (0/1, SMC_MIXED handles, default 1): run each of those
 * FGMRES solves in one persistent cooperative kernel on the device (1) or
 * with host-side control per iteration (0).
 * "inner_rtol_floor" (0 < f < 1): smallest relative tolerance asked of an
 * FP32 inner solve of the mixed form, for the Stokes and the temperature
 * solves; "stokes_inner_rtol_floor" (default 1e-3) and
 * "theta_inner_rtol_floor" (default 1e-4) set one of them.  The FP32
 * operator's rounding limits what an outer pass gains (about 2e-2 for the
 * Stokes operator at a 1e3 viscosity contrast), so a tighter inner solve
 * only adds Arnoldi steps.
 * "theta_precond_lag" (0 <= f < 1, default 0.3): the mixed form reuses the
 * temperature preconditioner while a0 stays within this relative distance
 * of the a0 it was built for (0: rebuild for every new a0, as the reference).
 * "bfbt_reuse_rel" (0 <= f < 1, default 0.02), "bfbt_reuse_age" (>= 1,
 * default 32): the mixed form keeps its BFBT blocks while the harmonic-mean
 * profile stays within this max-norm relative distance of the one they were
 * built from, for at most this many solves (set before the first Stokes solve).
 * "engine_ctas" (>= 0): the CTAs of the persistent Krylov engine, for handles
 * that share the GPU concurrently; default 0 = Nk R CTAs, R the smallest
 * count that leaves at most two z-points of the x-direction phase to a CTA,
 * capped at the co-resident maximum (one or two CTAs per SM).
 * "engine_phase_profile" (0/1, default 0): while the profiler is on, add the
 * engine's time between grid barriers, per phase, as profile regions named
 * "engine_stokes.<phase>" / "engine_theta.<phase>" (SM cycles of one CTA at
 * the peak clock, so a lower bound on wall time).
 * "engine_batch" (0/1, SMC_MIXED handles, default 0): send the refinement
 * solves to the device's batcher, which runs the solves of many handles in
 * one cooperative launch (each on its own CTAs and group barrier) instead of
 * one launch per solve; for handles stepped concurrently from several host
 * threads (smc_march_many sets it).  "engine_batch_ctas" (>= 0): CTAs of one
 * batched solve (0: one per Fourier row, at least 32).
 * "engine_batch_hold_us" (>= 0, default 50; applies to the handle's device):
 * how long the oldest queued solve waits for others before a batch starts.
 * "engine_batch_refill" (0/1, default 1), "engine_batch_idle_us" (default
 * 200), "engine_batch_life_us" (default 20000): a running batch takes solves
 * queued after its launch into slots that have finished theirs, until a slot
 * has waited idle_us for one or the launch has lived life_us (per device).
 * "engine_batch_gpu_ctas" (>= 0, default 0 = the co-resident maximum): cap on
 * the CTAs of one batched launch (per device).
 * "tc_transforms" (0/1, default 0): the z-contractions of the transforms by
 * the basis operators on the tensor cores (tcgen05, bf16 Ozaki slices with
 * exact FP32 accumulation: FP64-accurate; Nz <= 128).
 * "warm_start" (0/1, SMC_MIXED handles, default 1): each refinement solve
 * starts from the previous solve's solution (the last Stokes unknown, the
 * last step's temperature) and its FP64 residual instead of from zero; the
 * stopping test ||b - A x|| <= rtol ||b|| is unchanged.  "warm_extrapolate"
 * (0..3, default 1): bit 0 extrapolates the Stokes guess linearly in time
 * from the last two solves, bit 1 the temperature guess from the last two
 * steps (off by default: such guesses stalled the FP32-refined temperature
 * solves on the headline march).
 * "tc_lu" (0/1, default 1): the trailing updates of the dense Schur LU
 * (the legacy route's lagged factor, stokes/lagged_stokes.py:274-300) on the
 * tensor cores, FP64-accurate by the same splitting; 0 = FP64 SIMT. */
int smc_set_option(smc_handle* h, const char* key, double value);

/* RBCImplicitTheta.reset_history (implicit_theta.py:601-606). */
int smc_reset_history(smc_handle* h);

/* The BDF2 history of the temperature step (implicit_theta.py:596-599,
 * 616-619): the previous (projected) state, the previous stream function,
 * the previous dt and whether it exists.  The reference does not save it;
 * with it a checkpointed march resumes with the same BDF2 step instead of a
 * backward-Euler restart.  (Nk, Nz) complex buffers; the const model keeps
 * no history (have_prev = 0). */
int smc_get_history(smc_handle* h, double* prev_out, double* psi_prev_out, int mem,
                    double* dt_prev, int* have_prev);
int smc_set_history(smc_handle* h, const double* prev, const double* psi_prev, int mem,
                    double dt_prev, int have_prev);

int smc_counters_get(smc_handle* h, smc_counters* out);

/* Sizes of the handle's arrays: Nk, Nx, Nz, Np (= 2 Nx). */
int smc_shape(smc_handle* h, int* Nk, int* Nx, int* Nz, int* Np);

/* The handle's CUDA stream (cudaStream_t), for callers that order their own
 * work after the handle's. */
void* smc_stream(smc_handle* h);

/* ------------------------------------------------------------- many runs
 * An ensemble of independent runs (uneven grids, viscosity models, Rayleigh
 * numbers) on one GPU.  The reference runs one model per Python process and
 * has no batch API; its driver loop per run is api.march_adaptive
 * (specmc/api.py:169-190) with the amplitude abort threshold AMP_LIMIT
 * (specmc/_numerics.py:139-140). */

/* smc_create for each of cfgs[0 .. nruns-1] -> out[0 .. nruns-1]; on a
 * failure every handle already made is destroyed and the error names the run. */
int smc_create_many(const smc_config* cfgs, int nruns, smc_handle** out);

enum smc_run_status {
  SMC_RUN_OK = 0,          /* marched its steps */
  SMC_RUN_AMPLITUDE = 1,   /* max|theta| passed amp_limit x its initial value; marched on */
  SMC_RUN_NONFINITE = 2,   /* the state went non-finite; stopped */
  SMC_RUN_ERROR = 3        /* a hard error; stopped (smc_march_many returns < 0) */
};

typedef struct smc_run_result {
  long long steps;
  double t, dt;            /* march clock and last step size */
  double amp0, amp;        /* max |theta| on the (Nx, Nz) grid at the start / last check */
  double seconds;          /* wall time of this run's march */
  int status;              /* enum smc_run_status */
  int reserved;
} smc_run_result;

/* March the resident states (smc_set_state) of nruns handles nsteps
 * CFL-limited steps each (production_dt + step, api.march_adaptive),
 * checking finiteness and amplitude every check_every steps.  `concurrency`
 * host threads take the runs in order, each run on its own handle's stream.
 * batched != 0: the SMC_MIXED handles send their Krylov refinement solves to
 * the device's batcher, which runs the solves of many runs in one
 * cooperative launch, each on its own CTAs (option "engine_batch"); plain
 * handles step as usual.  Every run gets a result; the call returns < 0 if
 * any run met a hard error (the message names the first). */
int smc_march_many(smc_handle* const* hs, int nruns, long long nsteps, double safety,
                   double dtmax, double amp_limit, int check_every, int concurrency,
                   int batched, smc_run_result* res);

/* Batcher statistics of `device` since the process started: cooperative
 * launches, solves and CTAs they ran (no reference counterpart). */
int smc_batch_stats(int device, long long* launches, long long* solves, long long* ctas);

/* Grid synthesis that allocates nothing (no counterpart in the reference,
 * which has no device memory at all).  For callers that cannot allocate
 * device memory -- code whose memory is owned by a fixed arena that forbids
 * foreign cudaMalloc calls, or time loops that cannot afford the device-wide
 * synchronisation cudaMalloc/cudaFree may cause -- and therefore cannot hold a
 * model handle.  Turns (Nx/2+1, Nz) complex coefficients `that_dev` (device
 * memory) into grid values `grid_dev` (device memory, (Nx, Nz) or, with
 * `padded` != 0, (2Nx, Nz) float64), exactly what smc_transform does for
 * SMC_GRID / SMC_SYNTH_PAD.  The intermediate per-mode values live in one
 * fixed library-wide device array of SMC_NOALLOC_MAX_MODES complex entries
 * (8 MiB, held by every GPU that loads the library until exit); requests with
 * (Nx/2+1)*Nz above that limit are rejected with an error.  Asynchronous on
 * `stream` (a cudaStream_t; NULL = the legacy default stream).  The first call
 * on a device looks the array's address up (no allocation); make that first
 * call before capturing a stream.  All calls share the array: calls that
 * overlap on the GPU race; order them on one stream. */
#define SMC_NOALLOC_MAX_MODES 524288
int smc_grid_noalloc(const double* that_dev, double* grid_dev, int Nx, int Nz,
                     int padded, void* stream);

/* Message of the last hard error on the calling thread ("" if none). */
const char* smc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* SPECMC_GB300_H */
