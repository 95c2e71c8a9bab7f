// Declarations of the Schur-operator, eta-pipeline and set-up helpers
// (smc_schur.cu) and of the small-operator helpers of smc_dense.cu.
#pragma once
#include "smc_internal.cuh"

namespace smc {

// viscosity law + window of one model (coupled_model.py:333-399)
struct EtaLaw {
  double L = 0.0;        // ln(deta_T)
  double Ts = 0.0;       // Arrhenius offset (0: exponential law)
  double lo = 1e-3, hi = 1e3;          // window
  double lo_eff = 0.0, hi_eff = 0.0;   // window with the 1e-12 dead-band
  double w = 0.0, ylo = 0.0, yhi = 0.0;// smooth half-width, ln lo, ln hi
  int z_mode = 0;        // 0: T = 1 - z + th ; 1: T = th
  // pV(L) law when pvV > 0: ln eta = -pvE T / (Ts (T + Ts)) + pvV (1 - z) / (T + Ts)
  double pvE = 0.0, pvV = 0.0;
};

// C_b = alpha A_b B_b for N x N row-major operands (batch stride 0 = shared)
void bgemm(const Ctx& c, bool a_cplx, const void* A, long long sa, bool b_cplx, const void* B,
           long long sb, void* C, long long sc, int N, int batch, double alpha);
// stats = {min T, max T, #T outside [0,1], #T outside [0,2], #eta outside the
//          dead-band window, #ln(eta) strictly inside a smooth band}; null:
// only the per-CTA partials in scratch (for eta_stats_apply)
void eta_law(const Ctx& c, const double* th, const double* z, int N, long long npts,
             const EtaLaw& law, double* eta, double* stats, double* scratch);
// counts = {#outside dead-band window, #inside smooth band}; applies the
// clamp unless count_only
void eta_window(const Ctx& c, double* eta, long long npts, const EtaLaw& law, int count_only,
                double* counts, double* scratch);
// dst = {min eta, max pointwise relative drift vs lag (0 when lag null)}; null
// dst: only the per-CTA partials in scratch (for eta_guard)
void min_and_drift(const Ctx& c, const double* eta, const double* lag, long long n, double* dst,
                   double* scratch);
// out_j = w_j / mean_i(1 / eta[i][j]) as a complex vector (imaginary part 0)
void harm_profile_rhs(const Ctx& c, const double* eta, int Nx, int N, const double* wq,
                      double2* out);
void cheb_mult_real(const Ctx& c, const double* a, double* M, int N);
void reduced_blocks(const Ctx& c, const double* DM, const double* M, const double* CommG,
                    const double* V, const double* kx, double* Pcm, int N, int Nk);
void tau_ops(const Ctx& c, const double* D2, const double* kx, double lam, double* Acm, int N,
             int Nk);
// G_k = A_k^{-1} P (row-major), P = identity with rows N-2, N-1 zeroed
void green_from_lu(const Ctx& c, const double* LUcm, const int* piv, double* G, int N, int Nk);

// counters of the viscosity pipeline kept on the device (the step reads none
// of them; the handle's counters add them in when read)
struct EtaCtrDev {
  long long n_T_out_of_range, n_clip_T, n_clip_eta, n_smooth_eta, n_clip_eta_proj,
      n_smooth_eta_proj;
  double max_T_excursion;
};
// after eta_law (stats null) on the padded grid, from its per-CTA partials:
// adds its statistics to ctr and applies the hard clamp iff the window is hard
// and some point lies outside its dead band
void eta_stats_apply(const Ctx& c, const double* part, double* eta, long long npts,
                     const EtaLaw& law, EtaCtrDev* ctr);
// positivity guard of a truncated field (coupled_model.py:451-496), decided on
// the device from min_and_drift's partials (dst null) of the same field: when
// min(eta) is not > 0, counts the points outside the dead-band window into ctr
// and applies the window (smooth: always, counting the points inside its bands;
// hard: iff any point is outside).  scratch must not overlap mpart.
void eta_guard(const Ctx& c, const double* mpart, double* eta, long long npts, const EtaLaw& law,
               EtaCtrDev* ctr, double* scratch);

// reuse of the spectral BFBT blocks, decided on the device: whether the held
// profile is valid, and its age in solves
struct BfbtHold {
  int valid, age;
};
// sets `cond` (a conditional node of the launching graph) to 0 and ages the
// held profile when it is valid, younger than max_age solves, and
// max_q |prof_q - held_q| <= rel max_q |held_q| (real parts, NaN entries
// ignored as the host's std::max ignores them); otherwise held = prof, age 1
// and cond = 1 (the rebuild runs)
void bfbt_decide(const Ctx& c, const double2* prof, double2* held, int N, int max_age, double rel,
                 BfbtHold* h, cudaGraphConditionalHandle cond);

}  // namespace smc
