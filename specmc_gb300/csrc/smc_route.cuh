// Declarations of the route kernels (smc_krylov.cu).
#pragma once
#include "smc_internal.cuh"

namespace smc {
void theta_combine(const Ctx& c, const double2* v, const double2* A, const double* D2,
                   const double* Vi, const double* V, const double* kx, double a0, double2* out,
                   int Nk, int N);
void schur_combine(const Ctx& c, const double2* t1, const double2* t2, const double2* t3,
                   const double2* t4, const double2* v, const double* D, const double* D2,
                   const double* V, const double* kx, double2* out, int Nk, int N);
void const_rhs(const Ctx& c, const double2* th, const double2* Nc, double dt, double2* out,
               long long n);
void theta_rhs(const Ctx& c, const double2* th, const double2* prev, const double2* psi,
               const double2* phi, const double* kx, double b0, double b1, double H, double2* b,
               int Nk, int N);
void extrapolate(const Ctx& c, const double2* a, const double2* b, double2* out, long long n);
void vec_div(const Ctx& c, const double2* in, double h, double2* out, long long n);
void mgs(const Ctx& c, const double2* V, int j, long long n, double2* w, double2* hout);
void krylov_update(const Ctx& c, double2* x, const double2* Z, const double2* y, int k,
                   long long n);
// scratch: 6 ceil(N / 8) doubles; ticket: a zeroed word of the handle's
// (the kernel leaves it zero)
void diagnostics_reduce(const Ctx& c, const double* ux, const double* uz, const double* th,
                        const double2* that0, const double* D, const double* V, const double* wq,
                        int Nx, int N, double* out, double* scratch, unsigned int* ticket);
}  // namespace smc
