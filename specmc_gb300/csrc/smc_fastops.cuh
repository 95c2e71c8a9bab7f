// Fused operators of the fast (mixed) form (smc_fastops.cu).
#pragma once
#include "smc_internal.cuh"

namespace smc {

// Schur matvec with precomputed folded operators (T = double or float)
template <class T>
struct FusedSchur {
  int Nk = 0, N = 0, Mz = 0, L = 0;
  const T *Zf = nullptr, *Z1 = nullptr, *Z2 = nullptr, *Z3 = nullptr;  // (Mz,N), Nk x (Mz,N)
  const T *Zi = nullptr, *D2Zi = nullptr, *DZi = nullptr;              // (N, Mz)
  const void* tw = nullptr;      // L twiddles, complex T
  const double* kx = nullptr;
  const double* V = nullptr;     // FP64 basis (tau rows)
  void* vbuf = nullptr;          // Nk*N complex T scratch (FP32 copy of the input)
};

// temperature matvec (T = double or float)
template <class T>
struct FusedTheta {
  int Nk = 0, N = 0, Np = 0;
  const T *V = nullptr, *VD = nullptr, *D2 = nullptr, *Vi = nullptr;  // (N, N)
  const void* tw = nullptr;      // Np twiddles, complex T
  const double* kx = nullptr;
  const double* V64 = nullptr;
};

// Fv, Hv: 4 * Nk * Mz complex (double2-sized) scratch
void fused_schur_matvec(const Ctx& c, const FusedSchur<double>& op, const double* E,
                        const double2* v, double2* out, void* Fv, void* Hv);
void fused_schur_matvec(const Ctx& c, const FusedSchur<float>& op, const float* E,
                        const double2* v, double2* out, void* Fv, void* Hv);
// X: 2 * Nk * N complex scratch, A: Nk * N complex scratch
void fused_theta_matvec(const Ctx& c, const FusedTheta<double>& op, const double* ux,
                        const double* uz, double a0, const double2* v, double2* out, void* X,
                        void* A);
void fused_theta_matvec(const Ctx& c, const FusedTheta<float>& op, const float* ux,
                        const float* uz, double a0, const double2* v, double2* out, void* X,
                        void* A);
// cooperative CGS2 Arnoldi step; part: 2 G (j+1) + G complex
void cgs2(const Ctx& c, const double2* V, int j, long long n, double2* w, double2* hout,
          double2* part);
// out[k] = alpha G_k r_k for Nk real N x N operators (block preconditioners)
void kgemv(const Ctx& c, const double* G, const double2* r, double2* out, int Nk, int N,
           double alpha);
void rgemm_batched(const Ctx& c, const double* A, long long sa, const double* B, long long sb,
                   double* C, long long sc, int M, int K, int Nc, int batch);
void to_float(const Ctx& c, const double* in, float* out, long long n);

}  // namespace smc
