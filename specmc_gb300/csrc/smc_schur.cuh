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
//          dead-band window, #ln(eta) strictly inside a smooth band}
void eta_law(const Ctx& c, const double* th, const double* z, int N, long long npts,
             const EtaLaw& law, double* eta, double* stats, double* scratch);
// counts = {#outside dead-band window, #inside smooth band}; applies the
// clamp unless count_only
void eta_window(const Ctx& c, double* eta, long long npts, const EtaLaw& law, int count_only,
                double* counts, double* scratch);
// dst = {min eta, max pointwise relative drift vs lag (0 when lag null)}
void min_and_drift(const Ctx& c, const double* eta, const double* lag, long long n, double* dst,
                   double* scratch);
void harm_profile_rhs(const Ctx& c, const double* eta, int Nx, int N, const double* wq,
                      double* out);
void cheb_mult_real(const Ctx& c, const double* a, double* M, int N);
void reduced_blocks(const Ctx& c, const double* DM, const double* M, const double* CommG,
                    const double* V, const double* kx, double* Pcm, int N, int Nk);
void tau_ops(const Ctx& c, const double* D2, const double* kx, double lam, double* Acm, int N,
             int Nk);
// G_k = A_k^{-1} P (row-major), P = identity with rows N-2, N-1 zeroed
void green_from_lu(const Ctx& c, const double* LUcm, const int* piv, double* G, int N, int Nk);

}  // namespace smc
