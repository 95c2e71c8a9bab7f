// The truncated anelastic liquid approximation (TALA) of the FP64 time step
// (smc_tala.cu): operators with the reference density rho_bar(z) =
// exp((1 - z) Di) and its log-slope a = -Di (specmc/physics/compressibility.py).
#pragma once
#include "smc_internal.cuh"

namespace smc {

// Green operators of L^(rho)_k = D2 - a D - k^2 with the Dirichlet rows
// (column-major, one N x N per k; stokes/stokes_tala.py:226-240)
void tala_green_ops(const Ctx& c, const double* D, const double* D2, const double* kx, double a,
                    double* Acm, int N, int Nk);
// temperature preconditioner D2 - diag(k^2 + lam rho_j) with the Dirichlet
// rows (column-major; core/implicit_theta.py:471-493)
void tala_theta_ops(const Ctx& c, const double* D2, const double* kx, double lam, const double* rho,
                    double* Acm, int N, int Nk);
// out = a0 Mrho v - (D2 v - k^2 v) - MrhoVi A, rows N-2, N-1 = v(0), v(1)
// (implicit_theta.py:372-383); A = the x-analysis of the advective product
void tala_theta_combine(const Ctx& c, const double2* v, const double2* A, const double* Mrho,
                        const double* MrhoVi, const double* D2, const double* V, const double* kx,
                        double a0, double2* out, int Nk, int N);
// b = Mrho (b0 th - b1 prev) on rows < N-2 (tau rows 0); row k = 0 += H rho_c
// (all N entries); + adiab; rows < N-2 += phi  (implicit_theta.py:403-444)
void tala_theta_rhs(const Ctx& c, const double2* th, const double2* prev, const double* Mrho,
                    const double* rho_c, const double2* adiab, const double2* phi, double b0,
                    double b1, double H, double2* b, int Nk, int N);
// out = rho_j uz [1 - Di (1 - z_j + th)] on the padded grid (implicit_theta.py:336-350)
void tala_adiabatic_grid(const Ctx& c, const double* uz, const double* th, const double* rho,
                         const double* z, double Di, double* out, long long npts, int N);
// ux /= rho_j, uz /= rho_j on an (Ng, N) grid (rbc_galerkin.py:368-371)
void grid_div_rho(const Ctx& c, double* ux, double* uz, const double* rho, long long npts, int N);
// out[k][n] = alpha (in[k][n] s[n])   (stokes_tala.py:338-339)
void scale_cols(const Ctx& c, const double2* in, const double* s, double alpha, double2* out,
                int Nk, int N);
// TALA Schur epilogue (stokes_tala.py:427-466): t = mult_eta(v), T_bp =
// mult_eta(k^p D^b G v) for (b, p) = (0,1) (0,2) (1,0) (1,1) (2,0);
// out = D2 t - 2a D t + (a^2 - k^2) t + sum over the A12 monomials, tau rows
void tala_schur_combine(const Ctx& c, const double2* t, const double2* T01, const double2* T02,
                        const double2* T10, const double2* T11, const double2* T20,
                        const double2* v, const double* D, const double* D2, const double* V,
                        const double* kx, double a, double2* out, int Nk, int N);
// dense TALA Schur matrix (column-major, stokes_tala.py:252-303) from the
// product matrices Md of eta; work: 5 (2 Nk - 1) N^2 complex
void assemble_schur_tala(const Ctx& c, const double2* Md, const double* D, const double* D2,
                         const double* G, const double* V, const double* kx, double a,
                         double2* A, int Nk, int N, double2* work);

}  // namespace smc
