// Pseudo-spectral mult_eta (smc_pseudo.cu).
#pragma once
#include "smc_internal.cuh"

namespace smc {

struct PsPlan {
  int Nk = 0, N = 0, Mz = 0, L = 0;
  const double* Zf = nullptr;    // (Mz, N): T_q at the Mz CGL points
  const double* Zi = nullptr;    // (N, Mz): first N coefficients of the interpolant
  const double2* tw = nullptr;   // L twiddles e^{2 pi i m / L}
};

struct PsJobs {
  const double2* f[4];
  double2* out[4];
  double sgn[4];
};

// E (L, Mz) real: the eta field of the two-sided x-modes of eta_c on the grid
void ps_eta_grid(const Ctx& c, const PsPlan& pl, const double2* eta_c, double2* work, double* E);
// out_b = mult_eta(f_b) for nb <= 4 fields; Fv, Hv: nb * Nk * Mz scratch
void ps_mult_eta(const Ctx& c, const PsPlan& pl, const double* E, const PsJobs& jobs, int nb,
                 double2* Fv, double2* Hv);

}  // namespace smc
