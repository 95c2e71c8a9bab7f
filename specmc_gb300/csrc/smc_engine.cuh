// Persistent on-device FGMRES of the fast form (smc_engine.cu).
#pragma once
#include "smc_internal.cuh"

namespace smc {

// Operator + preconditioner of one engine solve.  Arrays typed T (the
// working precision) are passed as void*; kind 0 = fused Schur matvec,
// kind 1 = fused temperature matvec.
struct EngineOps {
  int kind = 0;
  int Nk = 0, N = 0, Mz = 0, L = 0, Np = 0;
  // Schur operator (T)
  const void *Zf = nullptr, *Z1 = nullptr, *Z2 = nullptr, *Z3 = nullptr;
  const void *Zi = nullptr, *D2Zi = nullptr, *DZi = nullptr, *E = nullptr, *twS = nullptr;
  // temperature operator (T)
  const void *tV = nullptr, *tVD = nullptr, *tD2 = nullptr, *tVi = nullptr, *twT = nullptr;
  const void *ux = nullptr, *uz = nullptr;
  double a0 = 0.0;
  const void* kxT = nullptr;          // kx in T
  const double* kx = nullptr;         // kx in FP64
  const double* V64 = nullptr;        // FP64 basis (tau rows)
  // preconditioner: out = palpha * Gp_k in_k (FP64 per-k operators)
  const double* Gp = nullptr;
  double palpha = 1.0;
  // scratch (T complex): vT (Nk N), Fv/Hv (4 Nk Mz), X (2 Nk N), A (Nk N)
  void *vT = nullptr, *Fv = nullptr, *Hv = nullptr, *X = nullptr, *A = nullptr;
};

struct EngineIO {
  const double2* b = nullptr;
  double2* x = nullptr;
  double rtol = 1e-8;
  int restart = 40, maxiter = 200;
  long long n = 0;
  double2 *V = nullptr, *Z = nullptr, *w = nullptr, *r = nullptr;
  double2* H = nullptr;      // (restart+1) x restart, column-major
  double2 *g = nullptr, *sn = nullptr, *y = nullptr;
  double* cs = nullptr;
  double2* part = nullptr;   // 2 * max_grid * (restart + 1)
  double* npart = nullptr;   // max_grid
  int* flag = nullptr;
  int* result = nullptr;     // {info, iterations}
  int max_grid = 0;
};

void fgmres_engine(const Ctx& c, const EngineOps& op, const EngineIO& io, bool fp32);

}  // namespace smc
