// Native runtime of the GB300 time step: model handles, device buffers, the
// control flow of the three SpecMC routes and the C ABI of include/specmc_gb300.h.
//
// Routes (the recipe each ConvectionConfig is translated into):
//   const  -> rbc_galerkin.RBC            explicit advection + BE diffusion
//   eta_z  -> implicit_theta.RBCImplicitTheta   frozen eta(z) Stokes + BDF2 theta
//   eta_T  -> coupled_model.RBCCoupled    eta(T) coupled Stokes + BDF2 theta
// Control decisions (FGMRES convergence, defect-correction stopping, refresh
// triggers, memo hits) are taken on the host from scalars the kernels reduce,
// exactly where the reference takes them; all vector and matrix work stays
// on the device, on the handle's stream.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <functional>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>
#include <set>
#include <mutex>
#include <thread>

#include "../../include/specmc_gb300.h"
#include "smc_internal.cuh"
#include "smc_route.cuh"
#include "smc_schur.cuh"
#include "smc_pseudo.cuh"
#include "smc_fastops.cuh"
#include "smc_engine.cuh"
#include "smc_batch.cuh"
#include "smc_tc.cuh"
#include "smc_tala.cuh"

namespace smc {

using cplx = std::complex<double>;
static thread_local std::string g_last_error;
void set_last_error(const char* msg) { g_last_error = msg ? msg : ""; }

// --------------------------------------------------------------- host basis
// CGL nodes, Chebyshev Vandermonde (chebvander recurrence), derivative
// (exact integers), inverse Vandermonde, Clenshaw-Curtis weights
// (rbc_galerkin.py:63-81, :284-287).
struct HostBasis {
  int N = 0;
  std::vector<double> z, V, Vi, D, D2, wq, VD, VD2, VT;

  static void host_inverse(const std::vector<double>& A, std::vector<double>& Ai, int N) {
    // Gauss-Jordan with partial pivoting (set-up only)
    std::vector<double> M(A);
    Ai.assign((size_t)N * N, 0.0);
    for (int i = 0; i < N; ++i) Ai[(size_t)i * N + i] = 1.0;
    for (int c = 0; c < N; ++c) {
      int p = c;
      for (int r = c + 1; r < N; ++r)
        if (std::fabs(M[(size_t)r * N + c]) > std::fabs(M[(size_t)p * N + c])) p = r;
      if (p != c)
        for (int q = 0; q < N; ++q) {
          std::swap(M[(size_t)c * N + q], M[(size_t)p * N + q]);
          std::swap(Ai[(size_t)c * N + q], Ai[(size_t)p * N + q]);
        }
      double piv = M[(size_t)c * N + c];
      if (piv == 0.0) throw std::runtime_error("singular Chebyshev Vandermonde");
      for (int q = 0; q < N; ++q) { M[(size_t)c * N + q] /= piv; Ai[(size_t)c * N + q] /= piv; }
      for (int r = 0; r < N; ++r) {
        if (r == c) continue;
        double f = M[(size_t)r * N + c];
        if (f == 0.0) continue;
        for (int q = 0; q < N; ++q) {
          M[(size_t)r * N + q] -= f * M[(size_t)c * N + q];
          Ai[(size_t)r * N + q] -= f * Ai[(size_t)c * N + q];
        }
      }
    }
  }

  explicit HostBasis(int N_) : N(N_) {
    z.resize(N);
    for (int j = 0; j < N; ++j) z[j] = 0.5 * (1.0 - std::cos(M_PI * j / (N - 1)));
    V.assign((size_t)N * N, 0.0);
    for (int j = 0; j < N; ++j) {
      double x = 2.0 * z[j] - 1.0, x2 = 2.0 * x;
      V[(size_t)j * N + 0] = 1.0;
      if (N > 1) V[(size_t)j * N + 1] = x;
      for (int k = 2; k < N; ++k)
        V[(size_t)j * N + k] = V[(size_t)j * N + k - 1] * x2 - V[(size_t)j * N + k - 2];
    }
    D.assign((size_t)N * N, 0.0);
    for (int k = 1; k < N; ++k)
      for (int n = k - 1; n >= 0; n -= 2) D[(size_t)n * N + k] = (n == 0 ? 2.0 : 4.0) * k;
    auto mm = [&](const std::vector<double>& A, const std::vector<double>& B) {
      std::vector<double> C((size_t)N * N, 0.0);
      for (int i = 0; i < N; ++i)
        for (int k = 0; k < N; ++k) {
          double a = A[(size_t)i * N + k];
          if (a == 0.0) continue;
          for (int j = 0; j < N; ++j) C[(size_t)i * N + j] += a * B[(size_t)k * N + j];
        }
      return C;
    };
    D2 = mm(D, D);
    host_inverse(V, Vi, N);
    std::vector<double> gk(N, 0.0);
    for (int k = 0; k < N; ++k) gk[k] = (k % 2) ? 0.0 : 1.0 / (1.0 - (double)k * k);
    gk[0] = 1.0;
    wq.assign(N, 0.0);
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < N; ++k) wq[j] += Vi[(size_t)k * N + j] * gk[k];
    VD = mm(V, D);
    VD2 = mm(V, D2);
    VT.assign((size_t)N * N, 0.0);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) VT[(size_t)j * N + i] = V[(size_t)i * N + j];
  }
};

// inverse of a dense row-major n x n matrix by Gauss-Jordan elimination with
// partial pivoting (set-up only)
static std::vector<double> invert_dense(std::vector<double> A, int n) {
  std::vector<double> X((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) X[(size_t)i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(A[(size_t)r * n + c]) > std::fabs(A[(size_t)p * n + c])) p = r;
    if (!(std::fabs(A[(size_t)p * n + c]) > 0.0)) throw std::runtime_error("invert_dense: singular matrix");
    if (p != c)
      for (int q = 0; q < n; ++q) {
        std::swap(A[(size_t)p * n + q], A[(size_t)c * n + q]);
        std::swap(X[(size_t)p * n + q], X[(size_t)c * n + q]);
      }
    const double inv = 1.0 / A[(size_t)c * n + c];
    for (int q = 0; q < n; ++q) { A[(size_t)c * n + q] *= inv; X[(size_t)c * n + q] *= inv; }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = A[(size_t)r * n + c];
      if (f == 0.0) continue;
      for (int q = 0; q < n; ++q) {
        A[(size_t)r * n + q] -= f * A[(size_t)c * n + q];
        X[(size_t)r * n + q] -= f * X[(size_t)c * n + q];
      }
    }
  }
  return X;
}

// ------------------------------------------------------------ device memory
// Every buffer is zeroed and every upload made on the handle's own stream:
// that stream is non-blocking, so work on the legacy default stream would not
// be ordered before the handle's kernels.
struct DevMem {
  std::vector<void*> ptrs;
  cudaStream_t s = nullptr;
  template <class T>
  T* alloc(size_t count) {
    void* p = nullptr;
    if (count == 0) count = 1;
    SMC_CUDA(cudaMalloc(&p, count * sizeof(T)));
    SMC_CUDA(cudaMemsetAsync(p, 0, count * sizeof(T), s));
    ptrs.push_back(p);
    return static_cast<T*>(p);
  }
  template <class T>
  T* upload(const std::vector<T>& h) {
    T* p = alloc<T>(h.size());
    SMC_CUDA(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    SMC_CUDA(cudaStreamSynchronize(s));     // h may go out of scope
    return p;
  }
  ~DevMem() {
    for (void* p : ptrs) cudaFree(p);
  }
};

struct LamSlot {
  double key = 0.0;
  double* LU = nullptr;
  int* piv = nullptr;
  double* Ginv = nullptr;   // A^{-1} P (tau columns zero): the solve as one GEMV
  float2* GinvT32 = nullptr;  // the same transposed per k ([k][m][n]) as (hi, lo) floats (engine)
  double* GinvT64 = nullptr;  // transposed, FP64 (engine)
  bool used = false;
};

struct FgmresResult {
  int info = 1;
  int iters = 0;
};

using Op = std::function<void(const double2*, double2*)>;

std::mutex& coop_mutex() {
  static std::mutex mu;
  return mu;
}

// the last cooperative launch per device (guarded by coop_mutex)
static cudaEvent_t g_coop_last[64] = {nullptr};
static bool g_coop_recorded[64] = {false};

void coop_order_before(cudaStream_t s) {
  int dev = 0;
  SMC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) throw std::runtime_error("cooperative launch: device ordinal >= 64");
  if (!g_coop_last[dev])
    SMC_CUDA(cudaEventCreateWithFlags(&g_coop_last[dev], cudaEventDisableTiming));
  if (g_coop_recorded[dev]) SMC_CUDA(cudaStreamWaitEvent(s, g_coop_last[dev], 0));
}

void coop_order_after(cudaStream_t s) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || !g_coop_last[dev]) return;
  if (cudaEventRecord(g_coop_last[dev], s) == cudaSuccess) g_coop_recorded[dev] = true;
}

void allow_max_smem(const void* f) {
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done;
  int dev = 0;
  SMC_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  if (done.count({f, dev})) return;
  int mx = 0;
  SMC_CUDA(cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  SMC_CUDA(cudaFuncGetAttributes(&fa, f));
  SMC_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                mx - (int)fa.sharedSizeBytes));
  done.insert({f, dev});
}

// ---------------------------------------------------------------- profiler
int Profiler::tag_of(const char* name) {
  for (int t = 0; t < MAXTAG; ++t) {
    if (names[t] == nullptr) { names[t] = name; return t; }
    if (std::strcmp(names[t], name) == 0) return t;
  }
  return MAXTAG - 1;
}
void Profiler::begin(cudaStream_t s, int tag, cudaEvent_t* a) {
  if (npool == 0) { SMC_CUDA(cudaEventCreate(a)); }
  else *a = pool[--npool];
  SMC_CUDA(cudaEventRecord(*a, s));
  (void)tag;
}
void Profiler::end(cudaStream_t s, int tag, cudaEvent_t a, double w, int is_bytes) {
  cudaEvent_t b;
  if (npool == 0) { SMC_CUDA(cudaEventCreate(&b)); }
  else b = pool[--npool];
  SMC_CUDA(cudaEventRecord(b, s));
  if (npend == cap) {
    int nc = cap ? 2 * cap : 1024;
    Pending* np = new Pending[nc];
    for (int i = 0; i < npend; ++i) np[i] = pend[i];
    delete[] pend;
    pend = np;
    cap = nc;
    cudaEvent_t* pp = new cudaEvent_t[2 * nc];
    for (int i = 0; i < npool; ++i) pp[i] = pool[i];
    delete[] pool;
    pool = pp;
  }
  pend[npend++] = Pending{tag, a, b};
  launches[tag]++;
  work[tag] += w;
  work_is_bytes[tag] = is_bytes;
}
void Profiler::resolve() {
  for (int i = 0; i < npend; ++i) {
    SMC_CUDA(cudaEventSynchronize(pend[i].b));
    float e = 0.f;
    SMC_CUDA(cudaEventElapsedTime(&e, pend[i].a, pend[i].b));
    ms[pend[i].tag] += e;
    pool[npool++] = pend[i].a;
    pool[npool++] = pend[i].b;
  }
  npend = 0;
}
void Profiler::add(const char* name, double ms_, long long n_) {
  const int t = tag_of(name);
  ms[t] += ms_;
  launches[t] += n_;
}
void Profiler::reset() {
  resolve();
  for (int t = 0; t < MAXTAG; ++t) { ms[t] = 0; launches[t] = 0; work[t] = 0; }
}
Profiler::~Profiler() {
  for (int i = 0; i < npend; ++i) { cudaEventDestroy(pend[i].a); cudaEventDestroy(pend[i].b); }
  for (int i = 0; i < npool; ++i) cudaEventDestroy(pool[i]);
  delete[] pend;
  delete[] pool;
}

// =================================================================== Model
struct Model {
  smc_config cfg{};
  int Nx = 0, N = 0, Nk = 0, Np = 0;
  long long n = 0, NN = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  long long nlaunch = 0;
  Ctx ctx;
  Profiler prof;
  // resident state of smc_set_state / smc_advance
  double t_resident = 0.0;
  bool resident_cur0 = true;
  DevMem mem;
  double* hbuf = nullptr;     // pinned scalars
  unsigned char* hpin = nullptr;   // pinned, 1 KB: engine results and phase counts
  static_assert(64 + ENGINE_PHASES * sizeof(long long) <= 256, "engine phase slots overlap");
  // pinned result slot of the refinement launches of kind k (0 Stokes, 1
  // temperature): int info, iterations, outer passes at +0, the final relative
  // residual at +16
  int* eng_slot_res(int k) const { return reinterpret_cast<int*>(hpin + 256 + 64 * k); }
  double* eng_slot_rel(int k) const { return reinterpret_cast<double*>(hpin + 256 + 64 * k + 16); }
  smc_counters ctr{};

  std::unique_ptr<HostBasis> hb;
  std::vector<double> kx_h, x_h;
  double dzmin = 0.0;
  // device basis
  double *dV, *dVi, *dD, *dD2, *dVD, *dVD2, *dVT, *dz, *dkx, *dwq;
  double2 *dtwNx, *dtwNp;
  int* dSkipK0;
  double *dLU0 = nullptr;   // tau lam = 0 (column-major)
  int* dPiv0 = nullptr;
  double* dG = nullptr;     // Green operators (row-major)
  LamSlot lam_slots[4];
  int lam_next = 0;
  // reduced operator (eta_z Stokes / BFBT blocks)
  double *dRedLU = nullptr;
  int* dRedPiv = nullptr;
  double *dM0, *dDM0, *dT1, *dT2, *dT3, *dComm, *dCommG, *dPcm;
  double* dMpLU = nullptr;
  int* dMpPiv = nullptr;
  double* dMpInv = nullptr;          // mixed form: explicit inverse, row-major
  // viscosity
  EtaLaw law;
  double *dEta = nullptr, *dEtaLag = nullptr, *dLastEta = nullptr, *dEtaP = nullptr,
         *dEtaPadZ = nullptr, *dZeroGrid = nullptr;
  double2 *dEtaC = nullptr, *dMd = nullptr, *dAsmWork = nullptr;
  double* dEzProf = nullptr;   // bounded depth profile eta(z) (eta_z / eta_T models)
  double2* dSchur = nullptr;
  int *dSchurPiv = nullptr, *dSchurPerm = nullptr;
  double2 *dSchurInvL = nullptr, *dSchurInvU = nullptr;
  bool have_lag = false;
  int n_since_refresh = 0;
  bool last_failed = false;
  // memo
  double2 *dMemoThat, *dMemoX, *dMemoPsi, *dMemoOm;
  bool memo_valid = false;
  // history
  double2 *dPrev, *dPsiPrev, *dPsiN;
  bool have_prev = false;
  double dt_prev = 0.0;
  double a0 = 1.0, b0 = 1.0, b1 = 0.0;
  // state and spectral work buffers
  double2 *dIn, *dOut, *dS0, *dS1, *dTh1, *dTh2, *dPsi, *dOm, *dPsiStar, *dRhs, *dPhi;
  double2* sp[16];
  double* gr[10];
  double *dRed, *dScal;
  // the viscosity pipeline's counters and the BFBT blocks' reuse state, kept
  // on the device so that no step waits on them
  EtaCtrDev* dEtaCtr = nullptr;
  unsigned int* dDiagTicket = nullptr;     // last-CTA ticket of the diagnostics reduction
  BfbtHold* dBfbtHold = nullptr;
  double2* dBfbtHeld = nullptr;
  // Krylov
  int mmax = 0;
  double2 *dKV, *dKZ, *dKw, *dKx, *dKr, *dKh, *dKy, *dKb;
  // Schur defect work
  double2 *dSb, *dSx, *dSr, *dSdx, *dSAx, *dSw, *dSf2, *dSf3, *dSf4, *dSt[4], *dSolveWork;
  double2 *dBfbtRhs, *dBfbtProfC;
  // TALA (compressibility SMC_TALA): rho_bar on the CGL nodes and its
  // inverse, the coefficients of rho_bar, product matrices of rho_bar and
  // rho_bar^2, Mrho Vi, the L^(rho) Green operators and work buffers
  bool tala = false;
  double tala_a = 0.0;
  double *dRho = nullptr, *dRhoInv = nullptr, *dRhoC = nullptr, *dMrho = nullptr,
         *dMrhoVi = nullptr, *dD2rho = nullptr, *dGt = nullptr;
  double2 *dTalaF = nullptr, *dTalaT = nullptr, *dTalaRhs = nullptr, *dTalaAd = nullptr;
  double *dTalaThG = nullptr, *dTalaAdG = nullptr;
  // the Green operators of the coupled Stokes operator (TALA: of L^(rho))
  const double* green_coupled() const { return tala ? dGt : dG; }
  // pseudo-spectral mult_eta
  PsPlan psplan;
  double* dPsE = nullptr;
  double2 *dPsFv = nullptr, *dPsHv = nullptr;
  bool use_dense_mult = false;
  // fast (mixed) form: BFBT-preconditioned FGMRES for the coupled Stokes
  // solve and explicit per-k inverse operators for the block preconditioners
  bool fast = false;
  double* dRedG = nullptr;
  float2* dRedGT32 = nullptr;      // transposed per k ([k][m][n]), (hi, lo) floats (engine)
  double* dRedGT64 = nullptr;      // transposed, FP64 (engine)
  FusedSchur<double> fs64;
  FusedSchur<float> fs32;
  // transposed operator matrices of the engine, per precision
  struct EngMats {
    const void *ZfT = nullptr, *Z1T = nullptr, *Z2T = nullptr, *Z3T = nullptr;
    const void *D2ZiT = nullptr, *ZiT = nullptr, *DZiT = nullptr;
    const void *tVT = nullptr, *tVDT = nullptr, *tD2T = nullptr, *tViT = nullptr;
    const void *ZfT2 = nullptr, *Z1T2 = nullptr, *D2ZiT2 = nullptr;   // (hi, lo) pairs (em32)
  } em32, em64;
  const float2* dev_transposed_split(const double* in, long long rows, long long cols, int batch) {
    float2* out = mem.alloc<float2>((size_t)rows * cols * batch);
    transpose_split(ctx, in, out, rows, cols, batch);
    return out;
  }
  template <class To>
  const To* dev_transposed(const double* in, long long rows, long long cols, int batch) {
    To* out = mem.alloc<To>((size_t)rows * cols * batch);
    transpose_as(ctx, in, out, rows, cols, batch);
    return out;
  }
  FusedTheta<double> ft64;
  FusedTheta<float> ft32;
  float *dE32 = nullptr, *dUx32 = nullptr, *dUz32 = nullptr;
  double2 *dFsFv = nullptr, *dFsHv = nullptr, *dFtX = nullptr, *dFtA = nullptr;
  double2 *dCgsPart = nullptr, *dRefR = nullptr, *dRefE = nullptr;
  long long n_outer = 0;
  int matvec_variant = 0;   // smc_schur_matvec: 0 plain, 1 fused FP64, 2 fused FP32
  bool inner_fp32 = true;   // fast form: FP32 inner Krylov operators + FP64 refinement
  // smallest relative tolerance asked of an FP32 inner solve: Stokes, temperature
  double inner_floor[2] = {1e-3, 1e-4};
  double theta_lag = 0.3;    // fast form: relative a0 change before the theta preconditioner is rebuilt
  long long n_theta_lag_hits = 0;
  long long n_fp64_fallback = 0;     // fast form: inner FP32 solves redone in FP64
  int stokes_fp64_solves = 0;        // fast form: Stokes solves left in FP64 after a fallback
  bool use_engine = true;   // fast form: Krylov solves in the persistent on-device engine
  EngineIO eio;
  float* dKx32 = nullptr;
  int* dEngInt = nullptr;
  bool eng_phase = false;            // per-phase cycle counts of engine solves into the profiler
  int eng_ctas = 0;                  // > 0: cap on the engine's CTAs (handles sharing the GPU)
  int eng_auto_ctas = 0;             // the engine's grid when eng_ctas is 0 (set in setup)
  long long* dEngPhase = nullptr;    // ENGINE_PHASES accumulators
  double* dEngRes = nullptr;         // final relative residual of a refinement launch
  double sm_khz = 0.0;               // peak SM clock (cycles -> ms)
  // batched mode: the refinement solves go to the device's batcher, which
  // runs the solves of many handles in one cooperative launch (smc_batch.cu)
  bool batch_mode = false;
  int batch_ctas = 0;                // CTAs of one solve in a batch (0: the default)
  EngineJobResult* hBatchRes = nullptr;   // host-mapped result block
  EngineJobResult* dBatchRes = nullptr;   // its device address
  cudaEvent_t batch_ready = nullptr;
  int batch_seq = 0;
  long long n_batched = 0;           // solves this handle ran through the batcher
  // tensor-core z-contractions (smc_tc.cu) of the basis operators
  std::unique_ptr<TcCache> tc_cache;

  void enable_tc(bool on) {
    if (on && N > TC_KMAX)
      throw std::runtime_error("tc_transforms needs Nz <= " + std::to_string(TC_KMAX));
    if (on && !tc_cache) {
      tc_cache.reset(new TcCache);
      tc_cache->K = N;
      tc_cache->err = mem.alloc<int>(1);
      for (const double* Z : {dV, dVi, dD, dD2, dVD, dVD2}) tc_cache->add(Z, N);
    }
    ctx.tc = on ? tc_cache.get() : nullptr;
  }
  // warm start of the mixed form's refinement solves: x enters holding the
  // previous solve's solution (the Stokes unknown of the last solve, the
  // temperature of the last step), and the first outer pass starts from its
  // FP64 residual instead of b; the stopping test ||b - A x|| <= rtol ||b|| is
  // the same, so the same tolerance is met from a closer start
  bool warm_start = true;
  // bit 0: the Stokes guess extrapolated linearly in time from the last two
  // solves (measured: 19% fewer BFBT iterations over the 200-step headline
  // march); bit 1: the temperature guess extrapolated from the last two steps
  // -- off: from such guesses the FP32-refined temperature solves stopped
  // converging within their budget (135 of 200 steps on the headline march,
  // which then diverged), while the previous step's temperature alone as the
  // guess converges as from zero
  int warm_extrap = 1;
  // extrapolated guesses: the Stokes unknown of the last two solves (one per
  // step) and the steps' dt, for a linear extrapolation in time
  double2 *dSxHist = nullptr, *dSxTmp = nullptr;
  long long steps_done = 0, sx_step = -1, sx_hist_step = -1;
  double step_dt[2] = {0.0, 0.0};        // dt of the last step, of the one before
  // x <- x + r (x - hist), r = dt_last / dt_before, when x and hist are the
  // solutions of the two steps just before (otherwise x alone)
  void stokes_guess(double2* x) {
    if (!warm_start) return;
    if (!dSxHist) { dSxHist = mem.alloc<double2>(n); dSxTmp = mem.alloc<double2>(n); }
    const long long cur = steps_done;
    const bool extrap = (warm_extrap & 1) && sx_step == cur - 1 && sx_hist_step == cur - 2 &&
                        step_dt[1] > 0.0;
    vec_copy(ctx, dSxTmp, x, n);                                  // x_n
    if (extrap) {
      const double r = step_dt[0] / step_dt[1];
      vec_axpby(ctx, x, make_double2(-r, 0.0), dSxHist, make_double2(1.0 + r, 0.0), n);
    }
    std::swap(dSxHist, dSxTmp);                                   // hist <- x_n
    sx_hist_step = sx_step;
    sx_step = cur;
  }
  // the dense Schur LU's trailing updates on the tensor cores (smc_tclu.cu):
  // on by default (FP64 accuracy; 2.4x / 4.1x faster factorisations at
  // 64x96 / 128x96 than the FP64 SIMT update); the option turns it off
  bool tc_lu = true;
  void* dTcLuWork = nullptr;
  int* dTcLuErr = nullptr;
  void enable_tc_lu(bool on) {
    tc_lu = on;
    if (on && !dTcLuErr) dTcLuErr = mem.alloc<int>(1);
  }
  // a tensor-core CTA that gave up waiting wrote NaN (contractions) or left
  // its tile alone (LU update) and raised a flag
  void check_tc() {
    for (int* flag : {tc_cache ? tc_cache->err : nullptr, dTcLuErr}) {
      if (!flag) continue;
      int e = 0;
      SMC_CUDA(cudaMemcpyAsync(hbuf, flag, sizeof(int), cudaMemcpyDeviceToHost, stream));
      SMC_CUDA(cudaStreamSynchronize(stream));
      std::memcpy(&e, hbuf, sizeof(int));
      if (e) {
        SMC_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), stream));
        throw std::runtime_error("tensor-core kernel: an mbarrier wait timed out");
      }
    }
  }

  void enable_batch(bool on) {
    if (on && !fast) throw std::runtime_error("engine_batch needs a SMC_MIXED handle");
    if (on && !hBatchRes) {
      SMC_CUDA(cudaHostAlloc((void**)&hBatchRes, sizeof(EngineJobResult), cudaHostAllocMapped));
      std::memset((void*)hBatchRes, 0, sizeof(EngineJobResult));
      SMC_CUDA(cudaHostGetDevicePointer((void**)&dBatchRes, (void*)hBatchRes, 0));
      SMC_CUDA(cudaEventCreateWithFlags(&batch_ready, cudaEventDisableTiming));
    }
    batch_mode = on;
  }

  // CTAs of one batched solve: a share of the GPU that lets several solves
  // run side by side -- one CTA per Fourier row, and at least 32
  int batch_grid(int kind) const {
    if (batch_ctas > 0) return batch_ctas;
    (void)kind;
    return std::max(32, std::min(Nk, 2 * ctx.num_sms));
  }

  // one refinement solve through the batcher: queue it, wait for its result
  FgmresResult batch_refine(int kind, const EngineOps& op32, const EngineOps& op64,
                            const EngineIO& io, const RefineIO& rf, double* true_res) {
    BatchReq r;
    r.job.op32 = op32;
    r.job.op64 = op64;
    r.job.io = io;
    r.job.rf = rf;
    r.job.out = dBatchRes;
    r.job.seq = ++batch_seq;
    r.G = std::min(batch_grid(kind), io.max_grid);
    r.smem = refine_engine_smem(op32, op64);
    r.ready = batch_ready;
    r.host = hBatchRes;
    hBatchRes->failed = 0;
    SMC_CUDA(cudaEventRecord(batch_ready, stream));
    batch_submit(device, &r);
    batch_wait(&r, 600.0);
    if (hBatchRes->failed)
      throw std::runtime_error(hBatchRes->failed == 1
                                   ? "batched engine: a group barrier timed out"
                                   : "batched engine: the batch could not be launched");
    ctx.count();
    ++n_batched;
    FgmresResult fr;
    fr.info = hBatchRes->info;
    fr.iters = hBatchRes->iters;
    n_outer += hBatchRes->outer;
    if (true_res) *true_res = hBatchRes->rel;
    return fr;
  }

  // ------------------------------------------------------------ utilities
  void sync_read(const double* d, int count) {
    SMC_CUDA(cudaMemcpyAsync(hbuf, d, count * sizeof(double), cudaMemcpyDeviceToHost, stream));
    SMC_CUDA(cudaStreamSynchronize(stream));
  }
  double norm(const double2* x) {
    vec_norm2(ctx, x, n, dScal, dRed);
    sync_read(dScal, 1);
    return hbuf[0];
  }

  // --------------------------------------------------------- transforms
  // values per mode X = f(k) * Zop @ cf, then x-synthesis on Ng points
  void synth(const double2* cf, const double* Zop, KFactor f, double* g, int Ng, double2* tmp) {
    ZJob j;
    j.Z = Zop; j.X = cf; j.Y = tmp; j.f = f;
    zmat_apply(ctx, &j, 1, Nk, N, dkx);
    SynthJob s{tmp, g};
    synth_x(ctx, &s, 1, Nk, N, Ng, Ng == Np ? dtwNp : dtwNx);
  }
  // grid (Ng) -> coefficients: Vi @ (rfft(g)/Ng)[:Nk]
  void analyze(const double* g, int Ng, double2* out, double2* tmp, KFactor f = KFactor(),
               int zero_tau = 0) {
    AnaJob a{g, tmp};
    analysis_x(ctx, &a, 1, Nk, N, Ng, Ng == Np ? dtwNp : dtwNx, 1.0 / Ng);
    ZJob j;
    j.Z = dVi; j.X = tmp; j.Y = out; j.f = f; j.zero_tau = zero_tau;
    zmat_apply(ctx, &j, 1, Nk, N, dkx);
  }
  void zop(const double* Z, long long zs, const double2* X, double2* Y, KFactor f = KFactor(),
           int x_real = 0, int accumulate = 0) {
    ZJob j;
    j.Z = Z; j.zstride = zs; j.X = X; j.Y = Y; j.f = f; j.x_real = x_real; j.accumulate = accumulate;
    zmat_apply(ctx, &j, 1, Nk, N, dkx);
  }

  // ------------------------------------------------------- LU lam cache
  // ChebTau factors keyed by round(lam, 10), at most 4 lam values
  // (rbc_galerkin.py:102,119-144)
  LamSlot& lam_lu(double lam) {
    double key = std::round(lam * 1e10) / 1e10;
    for (auto& s : lam_slots)
      if (s.used && s.key == key) return s;
    // fast form: the preconditioner of the temperature solve may lag a0 by
    // a small relative amount (the solve's residual is still enforced in FP64)
    if (fast && theta_lag > 0.0) {
      LamSlot* best = nullptr;
      for (auto& s : lam_slots)
        if (s.used && std::fabs(s.key - key) <= theta_lag * std::fabs(key) &&
            (!best || std::fabs(s.key - key) < std::fabs(best->key - key)))
          best = &s;
      if (best) { ++n_theta_lag_hits; return *best; }
    }
    int used = 0;
    for (auto& s : lam_slots) used += s.used;
    if (used >= 4)
      for (auto& s : lam_slots) s.used = false;
    LamSlot* slot = nullptr;
    for (auto& s : lam_slots)
      if (!s.used) { slot = &s; break; }
    ProfScope ps(ctx, "theta_lu_build");
    // TALA temperature step: D2 - diag(k^2 + lam rho_j) (implicit_theta.py:471-493);
    // the isoviscous model keeps the constant-coefficient ChebTau operator
    if (tala && cfg.model != SMC_MODEL_CONST) tala_theta_ops(ctx, dD2, dkx, lam, dRho, slot->LU, N, Nk);
    else tau_ops(ctx, dD2, dkx, lam, slot->LU, N, Nk);
    if (!fast) {
      lu_small_batched(ctx, slot->LU, slot->piv, nullptr, N, Nk);
    } else if (!lu_green_batched(ctx, slot->LU, slot->LU, slot->piv, slot->Ginv, slot->GinvT64,
                                 slot->GinvT32, N, Nk)) {
      lu_small_batched(ctx, slot->LU, slot->piv, nullptr, N, Nk);
      green_from_lu(ctx, slot->LU, slot->piv, slot->Ginv, N, Nk);
      transpose_split(ctx, slot->Ginv, slot->GinvT32, N, N, Nk);
      transpose_as(ctx, slot->Ginv, slot->GinvT64, N, N, Nk);
    }
    slot->key = key;
    slot->used = true;
    return *slot;
  }

  // ---------------------------------------------------------------- set-up
  void setup() {
    Nx = cfg.Nx; N = cfg.Nz; Nk = Nx / 2 + 1; Np = 2 * Nx;
    n = (long long)Nk * N; NN = (long long)N * N;
    SMC_CUDA(cudaSetDevice(cfg.device));
    device = cfg.device;
    SMC_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    mem.s = stream;
    int sms = 0;
    SMC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    ctx.s = stream; ctx.nlaunch = &nlaunch; ctx.num_sms = sms; ctx.prof = &prof;
    SMC_CUDA(cudaMallocHost(&hbuf, 4096 * sizeof(double)));
    SMC_CUDA(cudaMallocHost(&hpin, 1024));
    for (auto& e : eng_done) SMC_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    if (N < 4 || Nx < 4) throw std::runtime_error("Nx and Nz must be >= 4");

    hb.reset(new HostBasis(N));
    kx_h.resize(Nk);
    // 2 pi * rfftfreq(Nx, d=Lx/Nx) = 2 pi * (k * (1 / (Nx * (Lx/Nx))))
    const double fval = 1.0 / ((double)Nx * (cfg.Lx / Nx));
    for (int k = 0; k < Nk; ++k) kx_h[k] = (2.0 * M_PI) * ((double)k * fval);
    x_h.resize(Nx);
    for (int i = 0; i < Nx; ++i) x_h[i] = i * cfg.Lx / Nx;
    dzmin = INFINITY;
    for (int j = 0; j + 1 < N; ++j) dzmin = std::min(dzmin, hb->z[j + 1] - hb->z[j]);

    dV = mem.upload(hb->V); dVi = mem.upload(hb->Vi); dD = mem.upload(hb->D);
    dD2 = mem.upload(hb->D2); dVD = mem.upload(hb->VD); dVD2 = mem.upload(hb->VD2);
    dVT = mem.upload(hb->VT); dz = mem.upload(hb->z); dkx = mem.upload(kx_h);
    dwq = mem.upload(hb->wq);
    auto twiddles = [&](int Ng) {
      std::vector<double2> t(Ng);
      for (int m = 0; m < Ng; ++m) {
        long double a = 2.0L * (long double)M_PI * m / Ng;
        t[m] = make_double2((double)cosl(a), (double)sinl(a));
      }
      t[0] = make_double2(1.0, 0.0);
      if (Ng % 2 == 0) t[Ng / 2] = make_double2(-1.0, 0.0);
      if (Ng % 4 == 0) { t[Ng / 4] = make_double2(0.0, 1.0); t[3 * Ng / 4] = make_double2(0.0, -1.0); }
      return t;
    };
    dtwNx = mem.upload(twiddles(Nx));
    dtwNp = mem.upload(twiddles(Np));
    std::vector<int> skip(Nk, 0);
    for (int k = 0; k < Nk; ++k) skip[k] = (kx_h[k] == 0.0);
    dSkipK0 = mem.upload(skip);

    fast = cfg.precision == SMC_MIXED;
    for (auto& s : lam_slots) {
      s.LU = mem.alloc<double>(Nk * NN);
      s.piv = mem.alloc<int>(Nk * N);
      if (fast) {
        s.Ginv = mem.alloc<double>(Nk * NN);
        s.GinvT32 = mem.alloc<float2>(Nk * NN);
        s.GinvT64 = mem.alloc<double>(Nk * NN);
      }
    }
    dLU0 = mem.alloc<double>(Nk * NN);
    dPiv0 = mem.alloc<int>(Nk * N);
    dG = mem.alloc<double>(Nk * NN);

    dIn = mem.alloc<double2>(n); dOut = mem.alloc<double2>(n);
    dS0 = mem.alloc<double2>(n); dS1 = mem.alloc<double2>(n);
    dTh1 = mem.alloc<double2>(n); dTh2 = mem.alloc<double2>(n);
    dPsi = mem.alloc<double2>(n); dOm = mem.alloc<double2>(n);
    dPsiStar = mem.alloc<double2>(n); dRhs = mem.alloc<double2>(n); dPhi = mem.alloc<double2>(n);
    for (auto& p : sp) p = mem.alloc<double2>(n);
    for (auto& p : gr) p = mem.alloc<double>((size_t)Np * N);
    dRed = mem.alloc<double>(4096);
    dScal = mem.alloc<double>(64);
    dEtaCtr = mem.alloc<EtaCtrDev>(1);
    dDiagTicket = mem.alloc<unsigned int>(1);
    dPrev = mem.alloc<double2>(n); dPsiPrev = mem.alloc<double2>(n); dPsiN = mem.alloc<double2>(n);
    dMemoThat = mem.alloc<double2>(n); dMemoX = mem.alloc<double2>(n);
    dMemoPsi = mem.alloc<double2>(n); dMemoOm = mem.alloc<double2>(n);
    dZeroGrid = mem.alloc<double>((size_t)Np * N);

    // Stokes/Green factors at lam = 0 (every model factorises them at build)
    tau_ops(ctx, dD2, dkx, 0.0, dLU0, N, Nk);
    lu_small_batched(ctx, dLU0, dPiv0, nullptr, N, Nk);
    green_from_lu(ctx, dLU0, dPiv0, dG, N, Nk);
    if (cfg.compressibility == SMC_TALA) setup_tala();

    law.L = std::log(cfg.deta_T);
    law.Ts = cfg.model == SMC_MODEL_ETA_T ? cfg.arrhenius_Ts : 0.0;
    if (cfg.model == SMC_MODEL_ETA_T && cfg.arrhenius_V > 0.0) {
      law.pvE = cfg.arrhenius_E;
      law.pvV = cfg.arrhenius_V;
    }
    law.lo = cfg.eta_min; law.hi = cfg.eta_max;
    law.lo_eff = cfg.eta_min * (1.0 - 1e-12);
    law.hi_eff = cfg.eta_max * (1.0 + 1e-12);
    law.w = cfg.eta_smooth;
    law.ylo = std::log(cfg.eta_min); law.yhi = std::log(cfg.eta_max);

    if (cfg.model != SMC_MODEL_CONST) {
      mmax = std::max(cfg.theta_restart, cfg.stokes_restart);
      dKV = mem.alloc<double2>((size_t)(mmax + 1) * n);
      dKZ = mem.alloc<double2>((size_t)mmax * n);
      dKw = mem.alloc<double2>(n); dKx = mem.alloc<double2>(n); dKr = mem.alloc<double2>(n);
      dKb = mem.alloc<double2>(n);
      dKh = mem.alloc<double2>(mmax + 2); dKy = mem.alloc<double2>(mmax + 2);
      if (fast) {
        dCgsPart = mem.alloc<double2>((size_t)2 * sms * (mmax + 2) + sms + 64);
        dRefR = mem.alloc<double2>(n);
        dRefE = mem.alloc<double2>(n);
        setup_fused_theta();
        // persistent-engine workspace
        const int mr = mmax + 1, gmax = 2 * sms;
        eio.max_grid = gmax;
        eio.H = mem.alloc<double2>((size_t)mr * mr);
        eio.g = mem.alloc<double2>(mr + 1);
        eio.sn = mem.alloc<double2>(mr + 1);
        eio.y = mem.alloc<double2>(mr + 1);
        eio.cs = mem.alloc<double>(mr + 1);
        eio.part = mem.alloc<double2>((size_t)2 * gmax * (mr + 1));
        eio.npart = mem.alloc<double>(2 * gmax);
        dEngInt = mem.alloc<int>(8);
        eio.flag = dEngInt;
        eio.result = dEngInt + 4;
        eio.V = dKV; eio.Z = dKZ; eio.w = dKw; eio.r = dKr;
        dEngPhase = mem.alloc<long long>(ENGINE_PHASES);
        dEngRes = mem.alloc<double>(2);
        {
          int khz = 0;
          SMC_CUDA(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, device));
          sm_khz = khz > 0 ? (double)khz : 2.0e6;
        }
        dKx32 = mem.alloc<float>(Nk);
        to_float(ctx, dkx, dKx32, Nk);
      }
      dRedLU = mem.alloc<double>(Nk * NN); dRedPiv = mem.alloc<int>(Nk * N);
      dRedG = mem.alloc<double>(Nk * NN);
      dRedGT32 = mem.alloc<float2>(Nk * NN);
      dRedGT64 = mem.alloc<double>(Nk * NN);
      dM0 = mem.alloc<double>(NN); dDM0 = mem.alloc<double>(NN);
      dT1 = mem.alloc<double>(NN); dT2 = mem.alloc<double>(NN); dT3 = mem.alloc<double>(NN);
      dComm = mem.alloc<double>(NN); dCommG = mem.alloc<double>(Nk * NN);
      dPcm = mem.alloc<double>(Nk * NN);
      // frozen eta(z) of the depth-only base (convection_modes.py:96-107)
      dEzProf = mem.alloc<double>(N);
      double* dEz = dEzProf;
      EtaLaw lz = law;
      lz.Ts = 0.0;
      eta_law(ctx, dZeroGrid, dz, N, N, lz, dEz, dScal, dRed);
      sync_read(dScal, 6);
      double clip = hbuf[4], band = hbuf[5];
      if (law.w > 0.0) { ctr.n_clip_eta = (long long)clip; ctr.n_smooth_eta = (long long)band; }
      else if (clip > 0) { eta_window(ctx, dEz, N, lz, 0, dScal, dRed); ctr.n_clip_eta = (long long)clip; }
      // tiled (Nx, N) eta(z) and its padded re-synthesis (dissipation source)
      dEtaPadZ = mem.alloc<double>((size_t)Np * N);
      {
        std::vector<double> ez(N);
        SMC_CUDA(cudaMemcpyAsync(ez.data(), dEz, N * sizeof(double), cudaMemcpyDeviceToHost, stream));
        SMC_CUDA(cudaStreamSynchronize(stream));
        std::vector<double> tiled((size_t)Nx * N);
        for (int i = 0; i < Nx; ++i)
          for (int j = 0; j < N; ++j) tiled[(size_t)i * N + j] = ez[j];
        double* dTiled = mem.upload(tiled);
        eta_pad_from_grid(dTiled, dEtaPadZ);
      }
      if (cfg.model == SMC_MODEL_ETA_Z) {
        // eta_c = Vi @ eta_grid, reduced operator LU per k (vv_stokes.py:240-279)
        double2* dEzc = mem.alloc<double2>(N);
        double2* dEzIn = mem.alloc<double2>(N);
        {
          std::vector<double> ez(N);
          SMC_CUDA(cudaMemcpyAsync(ez.data(), dEz, N * sizeof(double), cudaMemcpyDeviceToHost, stream));
          SMC_CUDA(cudaStreamSynchronize(stream));
          std::vector<double2> ec(N);
          for (int j = 0; j < N; ++j) ec[j] = make_double2(ez[j], 0.0);
          SMC_CUDA(cudaMemcpyAsync(dEzIn, ec.data(), N * sizeof(double2), cudaMemcpyHostToDevice, stream));
          SMC_CUDA(cudaStreamSynchronize(stream));
        }
        ZJob j; j.Z = dVi; j.X = dEzIn; j.Y = dEzc;
        zmat_apply(ctx, &j, 1, 1, N, dkx);
        build_reduced_lu(dEzc, dRedLU, dRedPiv);
      } else {
        // coupled: eta fields, Schur storage, assembly workspace
        dEta = mem.alloc<double>((size_t)Nx * N);
        dEtaLag = mem.alloc<double>((size_t)Nx * N);
        dLastEta = mem.alloc<double>((size_t)Nx * N);
        dEtaP = mem.alloc<double>((size_t)Np * N);
        dEtaC = mem.alloc<double2>(n);
        // the dense Schur route (legacy solve, rescue) is allocated on first
        // use: its factor is (Nk N)^2 complex entries
        {
          size_t free_b = 0, total_b = 0;
          SMC_CUDA(cudaMemGetInfo(&free_b, &total_b));
          dense_cap_bytes = 0.5 * (double)free_b;
        }
        if (!fast && cfg.precond != SMC_PRECOND_BFBT) ensure_dense();
        dSb = mem.alloc<double2>(n); dSx = mem.alloc<double2>(n); dSr = mem.alloc<double2>(n);
        dSdx = mem.alloc<double2>(n); dSAx = mem.alloc<double2>(n); dSw = mem.alloc<double2>(n);
        dSf2 = mem.alloc<double2>(n); dSf3 = mem.alloc<double2>(n); dSf4 = mem.alloc<double2>(n);
        for (auto& p : dSt) p = mem.alloc<double2>(n);
        dSolveWork = mem.alloc<double2>(n);
        // pseudo-spectral plan: L >= 3 Nk - 2 x-points, Mz = 2N - 1 CGL points
        // L: the first power of two >= 3 Nk - 2 (alias-free products of two
        // Nk-mode fields; a power of two for the radix-2 FFTs)
        psplan.Nk = Nk; psplan.N = N; psplan.Mz = 2 * N - 1;
        psplan.L = 1;
        while (psplan.L < 3 * Nk - 2) psplan.L <<= 1;
        // default engine grid: R CTAs per Fourier row, R the smallest count
        // that leaves at most two of the Mz z-points of the x-direction phase
        // to a CTA.  A small problem then runs on fewer CTAs than the GPU
        // holds, which makes its grid barriers and partial-sum reductions
        // cheaper (64x96: 99 CTAs, 17% less time per step than 304); the
        // launch caps it at the co-resident maximum.
        eng_auto_ctas = Nk * std::max(1, (psplan.Mz + 2 * Nk - 1) / (2 * Nk));
        {
          const int Mz = psplan.Mz, L = psplan.L;
          std::vector<double> Zf((size_t)Mz * N), Zi((size_t)N * Mz);
          const long double PI = 3.14159265358979323846264338327950288L;
          for (int sI = 0; sI < Mz; ++sI)
            for (int q = 0; q < N; ++q) {
              // T_q(-cos(pi s/(Mz-1))) = (-1)^q cos(pi q s/(Mz-1))
              long long r = ((long long)q * sI) % (2LL * (Mz - 1));
              long double v = cosl(PI * (long double)r / (Mz - 1));
              if (q & 1) v = -v;
              Zf[(size_t)sI * N + q] = (double)v;
            }
          for (int pI = 0; pI < N; ++pI)
            for (int sI = 0; sI < Mz; ++sI) {
              long double w = (sI == 0 || sI == Mz - 1) ? 0.5L : 1.0L;
              long double g = (pI == 0 || pI == Mz - 1) ? 2.0L : 1.0L;
              long long r = ((long long)pI * sI) % (2LL * (Mz - 1));
              long double t = cosl(PI * (long double)r / (Mz - 1));
              if (pI & 1) t = -t;
              Zi[(size_t)pI * Mz + sI] = (double)(2.0L / (Mz - 1) / g * w * t);
            }
          std::vector<double2> tw(L);
          for (int m = 0; m < L; ++m) {
            long double a = 2.0L * PI * m / L;
            tw[m] = make_double2((double)cosl(a), (double)sinl(a));
          }
          tw[0] = make_double2(1.0, 0.0);
          psplan.Zf = mem.upload(Zf);
          psplan.Zi = mem.upload(Zi);
          psplan.tw = mem.upload(tw);
          dPsE = mem.alloc<double>((size_t)L * Mz);
          dPsFv = mem.alloc<double2>((size_t)4 * Nk * Mz);
          dPsHv = mem.alloc<double2>((size_t)4 * Nk * Mz);
        }
        if (fast) setup_fused_schur();
        dBfbtRhs = mem.alloc<double2>(N);
        dBfbtProfC = mem.alloc<double2>(N);
        dBfbtHeld = mem.alloc<double2>(N);
        dBfbtHold = mem.alloc<BfbtHold>(1);
        // Galerkin mass matrix V^T W V and its LU (stokes/bfbt.py:74-84)
        std::vector<double> Mp(NN, 0.0);
        for (int a = 0; a < N; ++a)
          for (int b = 0; b < N; ++b) {
            double s = 0;
            for (int j = 0; j < N; ++j) s += hb->V[(size_t)j * N + a] * hb->wq[j] * hb->V[(size_t)j * N + b];
            Mp[(size_t)b * N + a] = s;   // column-major
          }
        dMpLU = mem.upload(Mp);
        dMpPiv = mem.alloc<int>(N);
        lu_small_batched(ctx, dMpLU, dMpPiv, nullptr, N, 1);
        // the mixed form applies M^{-1} as a GEMV (the profile only feeds the
        // BFBT preconditioner there; a one-CTA triangular solve of N = 96
        // costs ~200 us of serial FP64 latency per Stokes solve)
        if (fast) {
          std::vector<double> Mr(NN);
          for (int a = 0; a < N; ++a)
            for (int b = 0; b < N; ++b) Mr[(size_t)a * N + b] = Mp[(size_t)b * N + a];
          dMpInv = mem.upload(invert_dense(Mr, N));
        }
      }
    }
    SMC_CUDA(cudaStreamSynchronize(stream));
  }

  // The TALA reference state (physics/compressibility.py:138-227, gamma = 1;
  // core/rbc_galerkin.py:298-306): a = -Di, rho_bar = exp((1 - z) Di) (exactly
  // 1 at Di = 0), its coefficients Vi rho_bar ([1, 0, ...] at Di = 0) and those
  // of rho_bar^2; the product matrices Mrho, Mrho Vi (temperature equation)
  // and M(rho_bar^2) (buoyancy), and on the coupled model the Green operators
  // of L^(rho) = D2 - a D - k^2 (stokes/stokes_tala.py:226-240).
  void setup_tala() {
    tala = true;
    const double Di = cfg.dissipation_number;
    tala_a = -Di / 1.0;
    auto prof = [&](double d) {
      std::vector<double> r(N, 1.0);
      if (d != 0.0)
        for (int j = 0; j < N; ++j) r[j] = std::exp((1.0 - hb->z[j]) * d / 1.0);
      return r;
    };
    auto coef = [&](double d) {
      std::vector<double> c(N, 0.0);
      if (d == 0.0) { c[0] = 1.0; return c; }
      std::vector<double> r = prof(d);
      for (int p = 0; p < N; ++p) {
        double s = 0.0;
        for (int j = 0; j < N; ++j) s += hb->Vi[(size_t)p * N + j] * r[j];
        c[p] = s;
      }
      return c;
    };
    // exact truncated Chebyshev product matrix (stokes/vv_stokes.py:81-109)
    auto cheb_mult = [&](const std::vector<double>& a) {
      std::vector<double> M((size_t)N * N);
      for (int p = 0; p < N; ++p)
        for (int q = 0; q < N; ++q) {
          double s = 0.0;
          if (p >= q) s += a[p - q];
          if (p + q < N) s += a[p + q];
          if (p > 0 && q >= p) s += a[q - p];
          M[(size_t)p * N + q] = 0.5 * s;
        }
      return M;
    };
    std::vector<double> rho = prof(Di), rinv(N), rc = coef(Di), r2c = coef(2.0 * Di);
    for (int j = 0; j < N; ++j) rinv[j] = 1.0 / rho[j];
    std::vector<double> Mr = cheb_mult(rc), MrVi((size_t)N * N, 0.0);
    for (int p = 0; p < N; ++p)
      for (int m = 0; m < N; ++m) {
        const double a = Mr[(size_t)p * N + m];
        for (int q = 0; q < N; ++q) MrVi[(size_t)p * N + q] += a * hb->Vi[(size_t)m * N + q];
      }
    dRho = mem.upload(rho); dRhoInv = mem.upload(rinv); dRhoC = mem.upload(rc);
    dMrho = mem.upload(Mr); dMrhoVi = mem.upload(MrVi); dD2rho = mem.upload(cheb_mult(r2c));
    if (cfg.model != SMC_MODEL_CONST) {
      dTalaThG = mem.alloc<double>((size_t)Np * N);
      dTalaAdG = mem.alloc<double>((size_t)Np * N);
      dTalaAd = mem.alloc<double2>(n);
    }
    if (cfg.model == SMC_MODEL_ETA_T) {
      double* lu = mem.alloc<double>(Nk * NN);
      int* piv = mem.alloc<int>(Nk * N);
      dGt = mem.alloc<double>(Nk * NN);
      tala_green_ops(ctx, dD, dD2, dkx, tala_a, lu, N, Nk);
      lu_small_batched(ctx, lu, piv, nullptr, N, Nk);
      green_from_lu(ctx, lu, piv, dGt, N, Nk);
      dTalaF = mem.alloc<double2>(5 * n);
      dTalaT = mem.alloc<double2>(6 * n);
      dTalaRhs = mem.alloc<double2>(n);
    }
  }

  // reduced operator LU from real Chebyshev coefficients `coef` (complex
  // storage, imaginary part ignored): P_k = (D2 - k^2) M + 2 k^2 [D,[D,M]] G_k
  void build_reduced_lu(const double2* coef, double* LU, int* piv) {
    build_reduced_blocks(coef);
    SMC_CUDA(cudaMemcpyAsync(LU, dPcm, sizeof(double) * Nk * NN, cudaMemcpyDeviceToDevice, stream));
    lu_small_batched(ctx, LU, piv, nullptr, N, Nk);
  }
  // the reduced operators P_k (column-major) into dPcm
  void build_reduced_blocks(const double2* coef) {
    // extract the real coefficient vector into dT3 (scratch), then M0
    realpart(coef, dT3, N);
    cheb_mult_real(ctx, dT3, dM0, N);
    bgemm(ctx, false, dD2, 0, false, dM0, 0, dDM0, 0, N, 1, 1.0);   // D2 M
    bgemm(ctx, false, dM0, 0, false, dD, 0, dT1, 0, N, 1, 1.0);     // M D
    bgemm(ctx, false, dD, 0, false, dT1, 0, dT2, 0, N, 1, 1.0);     // D M D
    bgemm(ctx, false, dM0, 0, false, dD2, 0, dT3, 0, N, 1, 1.0);    // M D2
    comm_combine(dDM0, dT2, dT3, dComm, (long long)NN);              // D2M - 2DMD + MD2
    bgemm(ctx, false, dComm, 0, false, dG, NN, dCommG, NN, N, Nk, 1.0);
    reduced_blocks(ctx, dDM0, dM0, dCommG, dV, dkx, dPcm, N, Nk);
  }

  void realpart(const double2* in, double* out, int count);
  void comm_combine(const double* a, const double* b, const double* c, double* out, long long cnt);

  // padded re-synthesis of a (Nx, N) viscosity grid: G(coeffs(eta))
  // (physics/dissipation.py:359-362)
  void eta_pad_from_grid(const double* eta_grid, double* out) {
    analyze(eta_grid, Nx, sp[14], sp[15]);
    synth(sp[14], dV, KFactor(), out, Np, sp[15]);
  }

  // ------------------------------------------------ fast-form operators
  template <class T>
  T* dev_copy_as(const double* src, long long count) {
    if (std::is_same<T, double>::value) {
      T* p = mem.alloc<T>(count);
      SMC_CUDA(cudaMemcpyAsync(p, src, count * sizeof(double), cudaMemcpyDeviceToDevice, stream));
      return p;
    }
    float* p = mem.alloc<float>(count);
    to_float(ctx, src, p, count);
    return reinterpret_cast<T*>(p);
  }

  void setup_fused_theta() {
    for (int prec = 0; prec < 2; ++prec) {
      if (prec == 0) {
        ft64.Nk = Nk; ft64.N = N; ft64.Np = Np; ft64.kx = dkx; ft64.V64 = dV;
        ft64.V = dV; ft64.VD = dVD; ft64.D2 = dD2; ft64.Vi = dVi; ft64.tw = dtwNp;
      } else {
        ft32.Nk = Nk; ft32.N = N; ft32.Np = Np; ft32.kx = dkx; ft32.V64 = dV;
        ft32.V = dev_copy_as<float>(dV, NN); ft32.VD = dev_copy_as<float>(dVD, NN);
        ft32.D2 = dev_copy_as<float>(dD2, NN); ft32.Vi = dev_copy_as<float>(dVi, NN);
        ft32.tw = dev_copy_as<float>(reinterpret_cast<const double*>(dtwNp), 2LL * Np);
      }
    }
    em64.tVT = dev_transposed<double>(dV, N, N, 1);
    em64.tVDT = dev_transposed<double>(dVD, N, N, 1);
    em64.tD2T = dev_transposed<double>(dD2, N, N, 1);
    em64.tViT = dev_transposed<double>(dVi, N, N, 1);
    em32.tVT = dev_transposed<float>(dV, N, N, 1);
    em32.tVDT = dev_transposed<float>(dVD, N, N, 1);
    em32.tD2T = dev_transposed<float>(dD2, N, N, 1);
    em32.tViT = dev_transposed<float>(dVi, N, N, 1);
    dUx32 = mem.alloc<float>((size_t)Np * N);
    dUz32 = mem.alloc<float>((size_t)Np * N);
    dFtX = mem.alloc<double2>((size_t)2 * n);
    dFtA = mem.alloc<double2>(n);
  }

  void setup_fused_schur() {
    const int Mz = psplan.Mz, L = psplan.L;
    const long long MN = (long long)Mz * N;
    double* D2G = mem.alloc<double>(Nk * NN);
    double* DG = mem.alloc<double>(Nk * NN);
    bgemm(ctx, false, dD2, 0, false, dG, NN, D2G, NN, N, Nk, 1.0);
    bgemm(ctx, false, dD, 0, false, dG, NN, DG, NN, N, Nk, 1.0);
    double* Z1 = mem.alloc<double>(Nk * MN);
    double* Z2 = mem.alloc<double>(Nk * MN);
    double* Z3 = mem.alloc<double>(Nk * MN);
    rgemm_batched(ctx, psplan.Zf, 0, dG, NN, Z1, MN, Mz, N, N, Nk);
    rgemm_batched(ctx, psplan.Zf, 0, D2G, NN, Z2, MN, Mz, N, N, Nk);
    rgemm_batched(ctx, psplan.Zf, 0, DG, NN, Z3, MN, Mz, N, N, Nk);
    double* D2Zi = mem.alloc<double>(MN);
    double* DZi = mem.alloc<double>(MN);
    rgemm_batched(ctx, dD2, 0, psplan.Zi, 0, D2Zi, 0, N, N, Mz, 1);
    rgemm_batched(ctx, dD, 0, psplan.Zi, 0, DZi, 0, N, N, Mz, 1);
    fs64.Nk = Nk; fs64.N = N; fs64.Mz = Mz; fs64.L = L; fs64.kx = dkx; fs64.V = dV;
    fs64.Zf = psplan.Zf; fs64.Z1 = Z1; fs64.Z2 = Z2; fs64.Z3 = Z3;
    fs64.Zi = psplan.Zi; fs64.D2Zi = D2Zi; fs64.DZi = DZi; fs64.tw = psplan.tw;
    fs32.Nk = Nk; fs32.N = N; fs32.Mz = Mz; fs32.L = L; fs32.kx = dkx; fs32.V = dV;
    fs32.Zf = dev_copy_as<float>(psplan.Zf, MN);
    fs32.Z1 = dev_copy_as<float>(Z1, Nk * MN);
    fs32.Z2 = dev_copy_as<float>(Z2, Nk * MN);
    fs32.Z3 = dev_copy_as<float>(Z3, Nk * MN);
    fs32.Zi = dev_copy_as<float>(psplan.Zi, MN);
    fs32.D2Zi = dev_copy_as<float>(D2Zi, MN);
    fs32.DZi = dev_copy_as<float>(DZi, MN);
    fs32.tw = dev_copy_as<float>(reinterpret_cast<const double*>(psplan.tw), 2LL * L);
    fs32.vbuf = mem.alloc<float2>(n);
    em64.ZfT = dev_transposed<double>(psplan.Zf, Mz, N, 1);
    em64.Z1T = dev_transposed<double>(Z1, Mz, N, Nk);
    em64.Z2T = dev_transposed<double>(Z2, Mz, N, Nk);
    em64.Z3T = dev_transposed<double>(Z3, Mz, N, Nk);
    em64.D2ZiT = dev_transposed<double>(D2Zi, N, Mz, 1);
    em64.ZiT = dev_transposed<double>(psplan.Zi, N, Mz, 1);
    em64.DZiT = dev_transposed<double>(DZi, N, Mz, 1);
    em32.ZfT = dev_transposed<float>(psplan.Zf, Mz, N, 1);
    em32.Z1T = dev_transposed<float>(Z1, Mz, N, Nk);
    em32.Z2T = dev_transposed<float>(Z2, Mz, N, Nk);
    em32.Z3T = dev_transposed<float>(Z3, Mz, N, Nk);
    em32.D2ZiT = dev_transposed<float>(D2Zi, N, Mz, 1);
    em32.ZiT = dev_transposed<float>(psplan.Zi, N, Mz, 1);
    em32.DZiT = dev_transposed<float>(DZi, N, Mz, 1);
    em32.ZfT2 = dev_transposed_split(psplan.Zf, Mz, N, 1);
    em32.Z1T2 = dev_transposed_split(Z1, Mz, N, Nk);
    em32.D2ZiT2 = dev_transposed_split(D2Zi, N, Mz, 1);
    dE32 = mem.alloc<float>((size_t)L * Mz);
    dFsFv = mem.alloc<double2>((size_t)4 * Nk * Mz);
    dFsHv = mem.alloc<double2>((size_t)4 * Nk * Mz);
  }

  void schur_matvec_fast(const double2* v, double2* out, bool fp32) {
    if (fp32) {
      ProfScope ps(ctx, "schur_matvec_f32", schur_ps_flops(), 0);
      fused_schur_matvec(ctx, fs32, dE32, v, out, dFsFv, dFsHv);
    } else {
      ProfScope ps(ctx, "schur_matvec_f64", schur_ps_flops(), 0);
      fused_schur_matvec(ctx, fs64, dPsE, v, out, dFsFv, dFsHv);
    }
  }

  // algorithmic flops of one fused pseudo-spectral Schur matvec
  double schur_ps_flops() const {
    const double Mz = psplan.Mz, L = psplan.L, nk = Nk, nz = N;
    double per_field = 4.0 * nk * Mz * nz + 8.0 * L * Mz * (nk - 1) + 2.0 * L * Mz +
                       8.0 * nk * L * Mz;
    return 4.0 * per_field + 3.0 * 4.0 * nk * nz * Mz;
  }

  void theta_matvec_fast(const double2* v, double2* out, bool fp32) {
    if (fp32) {
      ProfScope ps(ctx, "theta_matvec_f32");
      fused_theta_matvec(ctx, ft32, dUx32, dUz32, a0, v, out, dFtX, dFtA);
    } else {
      ProfScope ps(ctx, "theta_matvec_f64");
      fused_theta_matvec(ctx, ft64, gr[0], gr[1], a0, v, out, dFtX, dFtA);
    }
  }

  // Algorithmic bytes of an engine solve of `its` Arnoldi steps: per step the
  // operator's matrices are read once (z-contraction, epilogue, x-direction
  // weights), the block preconditioner once, the x-direction scratch written
  // and read, and the Krylov vectors touched four times per basis vector held
  // (first-pass dots, update, second-pass dots, next-vector combination) plus
  // the new V and Z rows written.
  double engine_bytes(int kind, bool fp32, int its, int restart) const {
    const double t = fp32 ? 4.0 : 8.0, cx = 2.0 * t, n8 = (double)n;
    double mats, scratch;
    if (kind == 0) {
      const double Mz = psplan.Mz, L = psplan.L;
      mats = t * Mz * N * (1.0 + 3.0 * Nk) + t * 3.0 * Mz * N + t * L * Mz;
      scratch = cx * 4.0 * Nk * Mz * 3.0;
    } else {
      mats = t * 4.0 * N * N + t * 2.0 * Np * N;
      scratch = cx * (2.0 * Nk * N * 2.0 + Nk * N * 2.0);
    }
    const double prec = (fp32 ? 8.0 : 8.0) * Nk * (double)NN;
    double vec = 0.0;
    for (int j = 0; j < its; ++j) {
      const int held = (restart > 0 ? j % restart : j) + 1;
      vec += cx * n8 * (4.0 * held + 2.0) + 16.0 * n8;
    }
    return its * (mats + scratch + prec) + vec;
  }

  // one FGMRES solve in the persistent engine; kind 0 = Schur, 1 = theta
  EngineOps engine_ops(int kind, bool fp32, const void* GpT, double palpha) const {
    const EngMats& em = fp32 ? em32 : em64;
    EngineOps op;
    op.kind = kind; op.Nk = Nk; op.N = N; op.kx = dkx; op.V64 = dV;
    op.GpT = GpT; op.palpha = palpha;
    op.kxT = fp32 ? (const void*)dKx32 : (const void*)dkx;
    if (kind == 0) {
      op.Mz = psplan.Mz; op.L = psplan.L;
      op.ZfT = em.ZfT; op.Z1T = em.Z1T; op.Z2T = em.Z2T; op.Z3T = em.Z3T;
      op.D2ZiT = em.D2ZiT; op.ZiT = em.ZiT; op.DZiT = em.DZiT;
      op.ZfT2 = em.ZfT2; op.Z1T2 = em.Z1T2; op.D2ZiT2 = em.D2ZiT2;
      if (fp32) { op.E = dE32; op.twS = fs32.tw; }
      else { op.E = dPsE; op.twS = fs64.tw; }
      op.Fv = dFsFv; op.Hv = dFsHv;
    } else {
      op.Np = Np; op.a0 = a0;
      op.tVT = em.tVT; op.tVDT = em.tVDT; op.tD2T = em.tD2T; op.tViT = em.tViT;
      if (fp32) { op.twT = ft32.tw; op.ux = dUx32; op.uz = dUz32; }
      else { op.twT = ft64.tw; op.ux = gr[0]; op.uz = gr[1]; }
      op.X = dFtX; op.A = dFtA;
    }
    return op;
  }

  FgmresResult engine_solve(int kind, bool fp32, const double2* b, double2* x, double rtol,
                            int restart, int maxiter, const void* GpT, double palpha) {
    ProfScope ps(ctx, kind == 0 ? "engine_stokes" : "engine_theta", 0.0, 1);
    const EngineOps op = engine_ops(kind, fp32, GpT, palpha);
    EngineIO io = eio;
    io.b = b; io.x = x; io.rtol = rtol; io.n = n;
    io.restart = std::max(1, std::min(restart, mmax));
    io.maxiter = maxiter;
    io.grid_cap = eng_ctas > 0 ? eng_ctas : eng_auto_ctas;
    const bool phases = eng_phase && prof.enabled;
    if (phases) {
      SMC_CUDA(cudaMemsetAsync(dEngPhase, 0, ENGINE_PHASES * sizeof(long long), stream));
      io.phase_cycles = dEngPhase;
    }
    fgmres_engine(ctx, op, io, fp32);
    int* res = reinterpret_cast<int*>(hpin);                     // pinned: no staged copies
    long long* cyc = reinterpret_cast<long long*>(hpin + 64);
    SMC_CUDA(cudaMemcpyAsync(res, eio.result, 2 * sizeof(int), cudaMemcpyDeviceToHost, stream));
    if (phases)
      SMC_CUDA(cudaMemcpyAsync(cyc, dEngPhase, ENGINE_PHASES * sizeof(long long),
                               cudaMemcpyDeviceToHost, stream));
    SMC_CUDA(cudaStreamSynchronize(stream));
    if (phases)
      for (int q = 0; q < ENGINE_PHASES; ++q)
        prof.add(engine_phase_names[kind][q],
                 q == EP_TOTAL_NS ? (double)cyc[q] * 1e-6 : (double)cyc[q] / sm_khz, 1);
    FgmresResult fr;
    fr.info = res[0];
    fr.iters = res[1];
    ps.work = engine_bytes(kind, fp32, fr.iters, io.restart);
    return fr;
  }

  // The whole FP32-inner / FP64-outer refinement in one engine launch (the
  // device runs the outer loop of fgmres_refined below); -> (info, inner
  // Arnoldi steps), *true_res = final relative FP64 residual.
  // defer: the launch's results are read at a later synchronisation
  // (engine_result); the returned info is -1 and true_res is not written
  FgmresResult engine_refine(int kind, const double2* b, double2* x, double rtol, int maxiter,
                             int restart, const void* GpT32, const void* GpT64, double palpha,
                             double* true_res, bool defer = false) {
    ProfScope ps(ctx, kind == 0 ? "engine_stokes" : "engine_theta", 0.0, 1);
    const EngineOps op32 = engine_ops(kind, true, GpT32, palpha);
    const EngineOps op64 = engine_ops(kind, false, GpT64, palpha);
    EngineIO io = eio;
    io.n = n;
    io.restart = std::max(1, std::min(restart, mmax));
    io.grid_cap = eng_ctas > 0 ? eng_ctas : eng_auto_ctas;
    RefineIO rf;
    rf.b = b; rf.x = x; rf.r = dRefR; rf.e = dRefE;
    rf.rtol = rtol; rf.floor = inner_floor[kind]; rf.maxiter = maxiter; rf.res = dEngRes;
    rf.warm = warm_start ? 1 : 0;
    if (batch_mode) {
      FgmresResult fr = batch_refine(kind, op32, op64, io, rf, true_res);
      ps.work = engine_bytes(kind, true, fr.iters, io.restart);
      return fr;
    }
    const bool phases = eng_phase && prof.enabled;
    if (phases) {
      SMC_CUDA(cudaMemsetAsync(dEngPhase, 0, ENGINE_PHASES * sizeof(long long), stream));
      io.phase_cycles = dEngPhase;
    }
    fgmres_refine_engine(ctx, op32, op64, io, rf);
    int* res = eng_slot_res(kind);                               // pinned: no staged copies
    long long* cyc = reinterpret_cast<long long*>(hpin + 64);
    double* relp = eng_slot_rel(kind);
    SMC_CUDA(cudaMemcpyAsync(res, eio.result, 3 * sizeof(int), cudaMemcpyDeviceToHost, stream));
    SMC_CUDA(cudaMemcpyAsync(relp, dEngRes, sizeof(double), cudaMemcpyDeviceToHost, stream));
    if (defer && !phases) {
      SMC_CUDA(cudaEventRecord(eng_done[kind], stream));
      eng_pending[kind] = true;
      eng_pending_restart[kind] = io.restart;
      FgmresResult fr;
      fr.info = -1;
      return fr;
    }
    if (phases)
      SMC_CUDA(cudaMemcpyAsync(cyc, dEngPhase, ENGINE_PHASES * sizeof(long long),
                               cudaMemcpyDeviceToHost, stream));
    SMC_CUDA(cudaStreamSynchronize(stream));
    if (phases)       // the refinement slots count outer passes; total_ns is wall time
      for (int q = 0; q < ENGINE_PHASES; ++q)
        prof.add(engine_phase_names[kind][q],
                 q == EP_TOTAL_NS ? (double)cyc[q] * 1e-6 : (double)cyc[q] / sm_khz,
                 (q >= EP_REF_XUPD && q <= EP_REFINE) ? res[2] : 1);
    FgmresResult fr;
    fr.info = res[0];
    fr.iters = res[1];
    n_outer += res[2];
    if (true_res) *true_res = *relp;
    // inner solves plus one FP64 operator application per outer pass
    ps.work = engine_bytes(kind, true, fr.iters, io.restart) +
              res[2] * 2.0 * engine_bytes(kind, true, 1, io.restart);
    return fr;
  }
  // deferred refinement launches: their results, the event after the copies
  bool eng_pending[2] = {false, false};
  int eng_pending_restart[2] = {0, 0};
  cudaEvent_t eng_done[2] = {nullptr, nullptr};
  // the results of a deferred launch of `kind` (waits for its copies, which a
  // synchronisation of the stream has normally completed already)
  FgmresResult engine_result(int kind, double* true_res) {
    SMC_CUDA(cudaEventSynchronize(eng_done[kind]));
    eng_pending[kind] = false;
    const int* res = eng_slot_res(kind);
    FgmresResult fr;
    fr.info = res[0];
    fr.iters = res[1];
    n_outer += res[2];
    if (true_res) *true_res = *eng_slot_rel(kind);
    const int rs = eng_pending_restart[kind];
    prof.add_work(kind == 0 ? "engine_stokes" : "engine_theta",
                  engine_bytes(kind, true, fr.iters, rs) + res[2] * 2.0 * engine_bytes(kind, true, 1, rs));
    return fr;
  }

  // FGMRES as iterative refinement: inner FGMRES on the FP32 operator, outer
  // residual r = b - A x in FP64; stops when ||r|| <= rtol ||b||.  Returns
  // (info, inner iterations) and the final true relative residual.
  using InnerSolve = std::function<FgmresResult(const double2*, double2*, double, int)>;
  FgmresResult fgmres_refined(const Op& A64, const InnerSolve& inner, const double2* b,
                              double2* x, double rtol, int maxiter, double floor, double* true_res) {
    FgmresResult res;
    vec_zero(ctx, x, n * sizeof(double2));
    const double bn = norm(b);
    const double tol = rtol * bn;
    vec_copy(ctx, dRefR, b, n);
    double beta = bn;
    int total = 0;
    res.info = 1;
    for (int outer = 0; outer < 12; ++outer) {
      if (beta <= tol) { res.info = 0; break; }
      if (total >= maxiter) break;
      const double inner_rtol = std::max(0.3 * tol / beta, floor);
      FgmresResult fr = inner(dRefR, dRefE, inner_rtol, maxiter - total);
      total += fr.iters;
      if (fr.info == 3) { res.info = 3; break; }   // non-finite data in the inner solve
      vec_axpby(ctx, x, make_double2(1.0, 0.0), dRefE, make_double2(1.0, 0.0), n);
      A64(x, dRefR);
      vec_axpby(ctx, dRefR, make_double2(1.0, 0.0), b, make_double2(-1.0, 0.0), n);
      beta = norm(dRefR);
      n_outer++;
      if (!std::isfinite(beta)) { res.info = 3; break; }
      if (fr.iters == 0 && beta > tol) break;     // no progress possible
    }
    if (beta <= tol && res.info != 3) res.info = 0;
    res.iters = total;
    if (true_res) *true_res = beta / std::max(bn, 1e-300);
    return res;
  }

  // ------------------------------------------------------ stokes routes
  void stokes_const(const double2* th, double2* psi, double2* om) {
    KFactor f; f.cre = 0.0; f.cim = -cfg.Ra; f.kpow = 1;      // -i k Ra theta
    vec_scaled_modes(ctx, th, sp[0], Nk, N, f, dkx, 0, 1);
    lu_small_solve(ctx, dLU0, dPiv0, NN, sp[0], om, N, Nk, 1.0, 1, dSkipK0);
    lu_small_solve(ctx, dLU0, dPiv0, NN, om, psi, N, Nk, -1.0, 1, dSkipK0);
    ctr.n_stokes++;
  }

  void stokes_etaz(const double2* th, double2* psi, double2* om) {
    KFactor f; f.cre = 0.0; f.cim = cfg.Ra; f.kpow = 1;       // i k Ra theta
    vec_scaled_modes(ctx, th, sp[0], Nk, N, f, dkx, 1, 1);
    lu_small_solve(ctx, dRedLU, dRedPiv, NN, sp[0], sp[1], N, Nk, 1.0, 1, dSkipK0);
    zop(dG, NN, sp[1], psi);
    vec_axpby(ctx, om, make_double2(-1.0, 0.0), sp[1], make_double2(0.0, 0.0), n);
    ctr.n_stokes++;
  }

  // eta_of (coupled_model.py:401-496) -> dEta (Nx, N)
  void eta_of(const double2* th) {
    ProfScope ps(ctx, "eta_of");
    synth(th, dV, KFactor(), gr[0], Np, sp[0]);              // theta on 2 Nx points
    eta_law(ctx, gr[0], dz, N, (long long)Np * N, law, dEtaP, nullptr, dRed);
    // the T / eta counters and the hard window of the padded field (applied
    // iff some point lies outside its dead band), decided on the device
    eta_stats_apply(ctx, dRed, dEtaP, (long long)Np * N, law, dEtaCtr);
    AnaJob a{dEtaP, sp[1]};
    analysis_x(ctx, &a, 1, Nk, N, Np, dtwNp, 1.0 / Np);
    SynthJob s{sp[1], dEta};
    synth_x(ctx, &s, 1, Nk, N, Nx, dtwNx);
    min_and_drift(ctx, dEta, nullptr, (long long)Nx * N, nullptr, dRed);
    // positivity guard (coupled_model.py:451-496), gated on min(eta) <= 0
    // (its count partials after the min/drift partials: at most 2 x 120)
    eta_guard(ctx, dRed, dEta, (long long)Nx * N, law, dEtaCtr, dRed + 256);
  }

  // Md (dense blocks, for the Schur assembly) and the pseudo-spectral eta
  // grid from the current dEta: eta_c = coeffs(eta)
  void eta_operator() {
    ProfScope ps(ctx, "eta_operator");
    analyze(dEta, Nx, dEtaC, sp[2]);
    md_stale = true;
    if (dMd && (!fast || use_dense_mult)) md_current();
    ps_eta_grid(ctx, psplan, dEtaC, dPsFv, dPsE);
    if (fast) to_float(ctx, dPsE, dE32, (long long)psplan.L * psplan.Mz);
  }

  // ------------------------------------------------ dense Schur route storage
  bool md_stale = true;
  double dense_cap_bytes = 0.0;
  // bytes of the dense route: Md, assembly/LU workspace, factor, inverses
  double dense_bytes() const {
    const double blk = (double)(2 * Nk - 1) * NN * 16.0;
    const long long nblk = (n + 63) / 64;
    return (tala ? 6.0 : 5.0) * blk + (double)n * n * 16.0 + 2.0 * nblk * 64 * 64 * 16.0 + 8.0 * n;
  }
  bool dense_feasible() const { return dSchur || dense_bytes() <= dense_cap_bytes; }
  void ensure_dense() {
    if (dSchur) return;
    if (!dense_feasible())
      throw std::runtime_error("dense Schur route: the factor of (Nk Nz)^2 = " +
                               std::to_string((double)n * n) +
                               " complex entries does not fit in device memory; use the "
                               "BFBT route (precond = SMC_PRECOND_BFBT)");
    if (!dMd) dMd = mem.alloc<double2>((size_t)(2 * Nk - 1) * NN);
    dAsmWork = mem.alloc<double2>((size_t)(tala ? 5 : 4) * (2 * Nk - 1) * NN);
    dSchur = mem.alloc<double2>((size_t)n * n);
    dSchurPiv = mem.alloc<int>(n);
    dSchurPerm = mem.alloc<int>(n);
    const long long nblk = (n + 63) / 64;
    dSchurInvL = mem.alloc<double2>((size_t)nblk * 64 * 64);
    dSchurInvU = mem.alloc<double2>((size_t)nblk * 64 * 64);
  }
  // Md of the current eta (the dense mult_eta blocks)
  void md_current() {
    if (!dMd) dMd = mem.alloc<double2>((size_t)(2 * Nk - 1) * NN);
    if (md_stale) {
      build_mult_mats(ctx, dEtaC, dMd, Nk, N);
      md_stale = false;
    }
  }

  // FreeSchurOperator.matvec at the current Md (lagged_stokes.py:202-220)
  void schur_matvec(const double2* v, double2* out) {
    if (tala) { schur_matvec_tala(v, out); return; }
    // algorithmic work of the dense form: 4 mult_eta x (Nk^2 + Nk(Nk-1)/2) N^2
    // complex MACs (8 flops each)
    ProfScope ps(ctx, "schur_matvec", 4.0 * 8.0 * ((double)Nk * Nk + 0.5 * Nk * (Nk - 1)) * NN, 0);
    zop(dG, NN, v, dSw);                                   // w = G v
    KFactor f2; f2.cre = 2.0; f2.kpow = 2;                  // 2 k^2 w
    vec_scaled_modes(ctx, dSw, dSf2, Nk, N, f2, dkx, 0, 0);
    zop(dD2, 0, dSw, dSf3);                                // D2 w
    KFactor f4; f4.kpow = 1;                                // k (D w)
    zop(dD, 0, dSw, dSf4, f4);
    if (use_dense_mult) {
      md_current();
      smc::mult_eta(ctx, dMd, v, dSt[0], Nk, N, -1.0, nullptr);
      smc::mult_eta(ctx, dMd, dSf2, dSt[1], Nk, N, -1.0, nullptr);
      smc::mult_eta(ctx, dMd, dSf3, dSt[2], Nk, N, -1.0, nullptr);
      smc::mult_eta(ctx, dMd, dSf4, dSt[3], Nk, N, +1.0, nullptr);
    } else {
      PsJobs j;
      j.f[0] = v; j.f[1] = dSf2; j.f[2] = dSf3; j.f[3] = dSf4;
      for (int q = 0; q < 4; ++q) j.out[q] = dSt[q];
      j.sgn[0] = j.sgn[1] = j.sgn[2] = -1.0;   // partner_sign
      j.sgn[3] = +1.0;                          // cross term: flipped
      ps_mult_eta(ctx, psplan, dPsE, j, 4, dPsFv, dPsHv);
    }
    schur_combine(ctx, dSt[0], dSt[1], dSt[2], dSt[3], v, dD, dD2, dV, dkx, out, Nk, N);
  }

  // TalaFreeOperator.matvec (stokes/stokes_tala.py:402-466): t = mult_eta(v)
  // and one mult_eta per distinct (D^b, k^p) image of g = G v, odd powers
  // of the input wavenumber with the flipped partner sign
  void schur_matvec_tala(const double2* v, double2* out) {
    ProfScope ps(ctx, "schur_matvec", 6.0 * 8.0 * ((double)Nk * Nk + 0.5 * Nk * (Nk - 1)) * NN, 0);
    zop(dGt, NN, v, dSw);                                  // g = G v
    double2* F01 = dTalaF;                                 // k g
    double2* F02 = dTalaF + n;                             // k^2 g
    double2* F10 = dTalaF + 2 * n;                         // D g
    double2* F11 = dTalaF + 3 * n;                         // k D g
    double2* F20 = dTalaF + 4 * n;                         // D2 g
    KFactor k1; k1.kpow = 1;
    KFactor k2; k2.kpow = 2;
    vec_scaled_modes(ctx, dSw, F01, Nk, N, k1, dkx, 0, 0);
    vec_scaled_modes(ctx, dSw, F02, Nk, N, k2, dkx, 0, 0);
    zop(dD, 0, dSw, F10);
    zop(dD, 0, dSw, F11, k1);
    zop(dD2, 0, dSw, F20);
    const double2* fin[6] = {v, F01, F02, F10, F11, F20};
    const double sgn[6] = {-1.0, +1.0, -1.0, -1.0, +1.0, -1.0};   // partner sign, flipped for odd k powers
    double2* T[6];
    for (int q = 0; q < 6; ++q) T[q] = dTalaT + q * n;
    if (use_dense_mult) {
      md_current();
      for (int q = 0; q < 6; ++q) smc::mult_eta(ctx, dMd, fin[q], T[q], Nk, N, sgn[q], nullptr);
    } else {
      for (int q0 = 0; q0 < 6; q0 += 4) {
        PsJobs j;
        const int nb = std::min(4, 6 - q0);
        for (int q = 0; q < nb; ++q) { j.f[q] = fin[q0 + q]; j.out[q] = T[q0 + q]; j.sgn[q] = sgn[q0 + q]; }
        ps_mult_eta(ctx, psplan, dPsE, j, nb, dPsFv, dPsHv);
      }
    }
    tala_schur_combine(ctx, T[0], T[1], T[2], T[3], T[4], T[5], v, dD, dD2, dV, dkx, tala_a, out,
                       Nk, N);
  }

  void rhs_schur(const double2* th, double2* b) {
    KFactor f; f.cre = 0.0; f.cim = cfg.Ra; f.kpow = 1;
    if (tala) {
      // i k Ra (rho_bar^2 theta) (stokes/stokes_tala.py:313-324)
      zop(dD2rho, 0, th, dTalaRhs);
      vec_scaled_modes(ctx, dTalaRhs, b, Nk, N, f, dkx, 1, 1);
      return;
    }
    vec_scaled_modes(ctx, th, b, Nk, N, f, dkx, 1, 1);
  }

  void refresh() {
    ensure_dense();
    md_current();
    {
      ProfScope ps(ctx, "schur_assembly");
      if (tala) assemble_schur_tala(ctx, dMd, dD, dD2, dGt, dV, dkx, tala_a, dSchur, Nk, N, dAsmWork);
      else assemble_schur(ctx, dMd, dD, dD2, dG, dV, dkx, dSchur, Nk, N, dAsmWork);
    }
    {
      // algorithmic work: complex LU, 8/3 n^3 real flops
      ProfScope ps(ctx, "schur_lu", 8.0 / 3.0 * (double)n * n * n, 0);
      if (tc_lu && !dTcLuErr) dTcLuErr = mem.alloc<int>(1);
      if (tc_lu && !dTcLuWork) dTcLuWork = mem.alloc<unsigned char>(tclu_work_bytes((int)n));
      zlu_dense(ctx, dSchur, dSchurPiv, (int)n, dAsmWork, tc_lu ? dTcLuWork : nullptr, dTcLuErr);
      zlu_diag_inverses(ctx, dSchur, (int)n, dSchurInvL, dSchurInvU);
    }
    std::vector<int> piv(n), perm(n);
    SMC_CUDA(cudaMemcpyAsync(piv.data(), dSchurPiv, n * sizeof(int), cudaMemcpyDeviceToHost, stream));
    SMC_CUDA(cudaStreamSynchronize(stream));
    for (long long i = 0; i < n; ++i) perm[i] = (int)i;
    for (long long i = 0; i < n; ++i) std::swap(perm[i], perm[piv[i]]);
    SMC_CUDA(cudaMemcpyAsync(dSchurPerm, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice, stream));
    SMC_CUDA(cudaMemcpyAsync(dEtaLag, dEta, sizeof(double) * Nx * N, cudaMemcpyDeviceToDevice, stream));
    SMC_CUDA(cudaStreamSynchronize(stream));
    have_lag = true;
    n_since_refresh = 0;
    ctr.n_refresh++;
  }

  void lag_solve(const double2* b, double2* x) {
    // algorithmic bytes: the n^2 complex factor is read once per solve
    ProfScope ps(ctx, "schur_lu_solve", 16.0 * (double)n * n, 1);
    zlu_dense_solve(ctx, dSchur, dSchurInvL, dSchurInvU, dSchurPerm, b, x, (int)n, dSolveWork);
  }

  // coupled_model.py:524-573
  void defect_solve(const double2* th, double2* x) {
    rhs_schur(th, dSb);
    lag_solve(dSb, x);
    double xn = std::max(norm(x), 1e-300);
    const bool adaptive = cfg.defect_tol > 0.0;
    const int kmax = adaptive ? cfg.max_K : cfg.K;
    int kdone = 0;
    double c = 0.0;
    for (int it = 0; it < kmax; ++it) {
      schur_matvec(x, dSAx);
      vec_axpby(ctx, dSAx, make_double2(1.0, 0.0), dSb, make_double2(-1.0, 0.0), n);  // r = b - Ax
      lag_solve(dSAx, dSdx);
      c = norm(dSdx) / xn;
      vec_axpby(ctx, x, make_double2(1.0, 0.0), dSdx, make_double2(1.0, 0.0), n);     // x += dx
      ++kdone;
      if (adaptive && c <= cfg.defect_tol) break;
    }
    // final residual of the accepted iterate (reported, as the reference does)
    schur_matvec(x, dSAx);
    vec_axpby(ctx, dSAx, make_double2(1.0, 0.0), dSb, make_double2(-1.0, 0.0), n);
    double bn = std::max(norm(dSb), 1e-300);
    ctr_last_defect_res = norm(dSAx) / bn;
    ctr.last_K = kdone;
    ctr.last_corr = kdone ? c : 0.0;
    ctr.n_defect++;
    if (!adaptive) last_failed = false;
    else {
      last_failed = !std::isfinite(ctr.last_corr) || ctr.last_corr > cfg.defect_tol;
      if (last_failed) ctr.n_defect_failed++;
    }
  }
  double ctr_last_defect_res = 0.0;

  void legacy_solve(const double2* th, double2* x) {
    double drift = INFINITY;
    if (have_lag) {
      min_and_drift(ctx, dEta, dEtaLag, (long long)Nx * N, dScal, dRed);
      sync_read(dScal, 2);
      drift = hbuf[1];
    }
    if (!have_lag || n_since_refresh >= cfg.lag || drift > cfg.eta_drift_tol) refresh();
    n_since_refresh++;
    defect_solve(th, x);
    if (last_failed) {
      refresh();
      n_since_refresh++;
      defect_solve(th, x);
      if (last_failed) ctr.n_defect_double_fail++;
    }
  }

  // spectral BFBT blocks from the harmonic-mean profile (stokes/bfbt.py:111-191).
  // The fast form keeps the blocks while the Galerkin profile stays within
  // 2% (max-norm, relative) of the one they were built from and for at most
  // 32 solves: the blocks only precondition, so the solution is unchanged.
  // The decision is taken on the device (bfbt_decide) inside a CUDA graph
  // whose rebuild runs under a conditional node the decision sets: one graph
  // launch per solve, the host enqueues the solve without waiting for it,
  // and a skipped rebuild launches none of its kernels.
  void bfbt_build() {
    ProfScope psp(ctx, "bfbt_profile");
    harm_profile_rhs(ctx, dEta, Nx, N, dwq, dBfbtRhs);
    ZJob j; j.Z = dVT; j.X = dBfbtRhs; j.Y = dBfbtProfC;     // V^T (w g)
    zmat_apply(ctx, &j, 1, 1, N, dkx);
    if (fast) kgemv(ctx, dMpInv, dBfbtProfC, dBfbtRhs, 1, N, 1.0);
    else lu_small_solve(ctx, dMpLU, dMpPiv, NN, dBfbtProfC, dBfbtRhs, N, 1, 1.0, 0, nullptr);
    ProfScope ps(ctx, "bfbt_build");
    if (!fast) {
      build_reduced_lu(dBfbtRhs, dRedLU, dRedPiv);
      return;
    }
    if (!bfbt_exec) bfbt_graph_make();
    SMC_CUDA(cudaGraphLaunch(bfbt_exec, stream));
    ctx.count();
  }
  // the fast form's blocks from dBfbtRhs: reduced operators, their LU, the
  // explicit inverses and the engine's transposed copies
  void bfbt_rebuild_launches() {
    build_reduced_blocks(dBfbtRhs);
    if (lu_green_batched(ctx, dPcm, dRedLU, dRedPiv, dRedG, dRedGT64, dRedGT32, N, Nk)) return;
    SMC_CUDA(cudaMemcpyAsync(dRedLU, dPcm, sizeof(double) * Nk * NN, cudaMemcpyDeviceToDevice, stream));
    lu_small_batched(ctx, dRedLU, dRedPiv, nullptr, N, Nk);
    green_from_lu(ctx, dRedLU, dRedPiv, dRedG, N, Nk);
    transpose_split(ctx, dRedG, dRedGT32, N, N, Nk);
    transpose_as(ctx, dRedG, dRedGT64, N, N, Nk);
  }
  cudaGraph_t bfbt_graph = nullptr;
  cudaGraphExec_t bfbt_exec = nullptr;
  // records f's launches on the stream into g (the capture ends on an
  // exception too, so the stream is usable afterwards)
  template <class F>
  void capture_into(cudaGraph_t g, F&& f) {
    SMC_CUDA(cudaStreamBeginCaptureToGraph(stream, g, nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal));
    try {
      f();
    } catch (...) {
      cudaGraph_t dummy = nullptr;
      cudaStreamEndCapture(stream, &dummy);
      throw;
    }
    cudaGraph_t out = nullptr;
    SMC_CUDA(cudaStreamEndCapture(stream, &out));
  }
  // graph: [bfbt_decide] -> IF (cond) { bfbt_rebuild_launches }
  void bfbt_graph_make() {
    SMC_CUDA(cudaGraphCreate(&bfbt_graph, 0));
    cudaGraphConditionalHandle cond;
    SMC_CUDA(cudaGraphConditionalHandleCreate(&cond, bfbt_graph, 0, cudaGraphCondAssignDefault));
    capture_into(bfbt_graph, [&] {
      bfbt_decide(ctx, dBfbtRhs, dBfbtHeld, N, bfbt_reuse_age, bfbt_reuse_rel, dBfbtHold, cond);
    });
    cudaGraphNode_t decide = nullptr;
    size_t nn = 1;
    SMC_CUDA(cudaGraphGetNodes(bfbt_graph, &decide, &nn));
    if (nn != 1) throw std::runtime_error("bfbt graph: expected one decision node");
    // zeroed storage: the struct's union has no default constructor
    alignas(cudaGraphNodeParams) unsigned char pbuf[sizeof(cudaGraphNodeParams)] = {};
    cudaGraphNodeParams& p = *reinterpret_cast<cudaGraphNodeParams*>(pbuf);
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = cond;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    SMC_CUDA(cudaGraphAddNode(&node, bfbt_graph, &decide, nullptr, 1, &p));
    capture_into(p.conditional.phGraph_out[0], [&] { bfbt_rebuild_launches(); });
    SMC_CUDA(cudaGraphInstantiate(&bfbt_exec, bfbt_graph, 0));
  }
  // reuse of the BFBT blocks: profile within bfbt_reuse_rel (max-norm,
  // relative) of the one they were built from, at most bfbt_reuse_age solves
  // (captured into the rebuild graph at the handle's first fast BFBT solve)
  int bfbt_reuse_age = 32;
  double bfbt_reuse_rel = 0.02;
  // the next build runs whatever the profile (held profile invalid)
  void bfbt_invalidate() {
    if (dBfbtHold) SMC_CUDA(cudaMemsetAsync(&dBfbtHold->valid, 0, sizeof(int), stream));
  }

  double schur_true_res(const double2* b, const double2* x) {
    schur_matvec(x, dSAx);
    vec_axpby(ctx, dSAx, make_double2(1.0, 0.0), b, make_double2(-1.0, 0.0), n);
    double bn = std::max(norm(b), 1e-300);
    return norm(dSAx) / bn;
  }

  // fast form, after a dense rescue (the BFBT blocks have just failed for
  // this eta field; the dense factor is fresh):
  //  lu_mode 1: FP64 FGMRES preconditioned by the lagged factor, which is not
  //    refactored however far eta drifts (the legacy route refactors at every
  //    drifted step: tens to hundreds of ms at 64x48..128x96), while solves
  //    converge within LU_PRECOND_SLOW iterations (then BFBT again); a solve
  //    that does not converge within LU_PRECOND_MAXIT (eta moves too fast for
  //    a stale factor) is solved by, and turns to,
  //  lu_mode 2: the legacy lagged-LU route (coupled_model.py:524-586,
  //    refactored as its drift test asks) for `lag` solves, then BFBT again.
  static constexpr int LU_PRECOND_MAXIT = 40, LU_PRECOND_SLOW = 20;
  int lu_mode = 0, legacy_left = 0;

  void bfbt_solve(const double2* th, double2* x) {
    rhs_schur(th, dSb);
    if (fast && lu_mode == 1 && dSchur && have_lag) {
      Op A64 = [&](const double2* v, double2* o) { schur_matvec_fast(v, o, false); };
      Op M = [&](const double2* r, double2* z) { lag_solve(r, z); };
      FgmresResult fr = fgmres(A64, M, dSb, x, cfg.stokes_rtol, cfg.stokes_restart, LU_PRECOND_MAXIT);
      schur_matvec_fast(x, dSAx, false);
      vec_axpby(ctx, dSAx, make_double2(1.0, 0.0), dSb, make_double2(-1.0, 0.0), n);
      const double res = norm(dSAx) / std::max(norm(dSb), 1e-300);
      if (fr.info == 0 || res <= cfg.stokes_rtol) {
        ctr.n_bfbt_solves++;
        ctr.n_bfbt_iters += fr.iters;
        ctr.last_bfbt_true_res = res;
        ctr.last_K = 0;
        if (fr.iters > LU_PRECOND_SLOW) lu_mode = 0;
        return;
      }
      lu_mode = 2;
      legacy_left = cfg.lag;
    }
    if (fast && lu_mode == 2 && dSchur) {
      if (--legacy_left <= 0) lu_mode = 0;
      legacy_solve(th, x);
      return;
    }
    bfbt_build();
    Op A = [&](const double2* v, double2* o) { schur_matvec(v, o); };
    Op M = [&](const double2* r, double2* z) {
      ProfScope ps(ctx, "bfbt_precond");
      if (fast) kgemv(ctx, dRedG, r, z, Nk, N, 1.0);      // (P_k^{-1} P) r
      else lu_small_solve(ctx, dRedLU, dRedPiv, NN, r, z, N, Nk, 1.0, 1, nullptr);
    };
    FgmresResult fr;
    double res;
    if (fast) {
      Op A64 = [&](const double2* v, double2* o) { schur_matvec_fast(v, o, false); };
      Op A32 = [&](const double2* v, double2* o) { schur_matvec_fast(v, o, true); };
      const bool fp32_now = inner_fp32 && stokes_fp64_solves == 0;
      if (!fp32_now && stokes_fp64_solves > 0) --stokes_fp64_solves;
      if (fp32_now) {
        if (use_engine) {
          stokes_guess(x);
          if (defer_stokes && !batch_mode && !(eng_phase && prof.enabled)) {
            // the host goes on enqueueing (velocity, CFL reduction) while
            // the engine runs; stokes_finish() completes this solve after
            // the CFL synchronisation
            engine_refine(0, dSb, x, cfg.stokes_rtol, cfg.stokes_maxiter, cfg.stokes_restart,
                          dRedGT32, dRedGT64, 1.0, nullptr, true);
            stokes_pend_th = th;
            stokes_pend_x = x;
            return;
          }
          fr = engine_refine(0, dSb, x, cfg.stokes_rtol, cfg.stokes_maxiter, cfg.stokes_restart,
                             dRedGT32, dRedGT64, 1.0, &res);
        } else {
          InnerSolve inner = [&](const double2* r, double2* e, double tol, int mi) {
            return fgmres(A32, M, r, e, tol, cfg.stokes_restart, mi);
          };
          fr = fgmres_refined(A64, inner, dSb, x, cfg.stokes_rtol, cfg.stokes_maxiter, inner_floor[0],
                              &res);
        }
        stokes_fp64_fallback(fr, res, x);
      } else {
        if (use_engine)
          fr = engine_solve(0, false, dSb, x, cfg.stokes_rtol, cfg.stokes_restart,
                            cfg.stokes_maxiter, dRedGT64, 1.0);
        else
          fr = fgmres(A64, M, dSb, x, cfg.stokes_rtol, cfg.stokes_restart, cfg.stokes_maxiter);
        schur_matvec_fast(x, dSAx, false);
        vec_axpby(ctx, dSAx, make_double2(1.0, 0.0), dSb, make_double2(-1.0, 0.0), n);
        res = norm(dSAx) / std::max(norm(dSb), 1e-300);
      }
    } else {
      fr = fgmres(A, M, dSb, x, cfg.stokes_rtol, cfg.stokes_restart, cfg.stokes_maxiter);
      res = schur_true_res(dSb, x);
    }
    bfbt_finish(th, x, fr, res);
  }

  // fast form: the FP32-refined solve did not reach the tolerance (viscosity
  // contrast too large for the FP32 operator's rounding): solve the system in
  // FP64 and stay in FP64 for the next 16 solves.  True when it ran.
  bool stokes_fp64_fallback(FgmresResult& fr, double& res, double2* x) {
    if (!(fr.info != 0 && !(res <= cfg.stokes_rtol))) return false;
    ctr.n_bfbt_iters += fr.iters;
    ++n_fp64_fallback;
    stokes_fp64_solves = 16;
    if (use_engine) {
      fr = engine_solve(0, false, dSb, x, cfg.stokes_rtol, cfg.stokes_restart, cfg.stokes_maxiter,
                        dRedGT64, 1.0);
    } else {
      Op A64 = [&](const double2* v, double2* o) { schur_matvec_fast(v, o, false); };
      Op M = [&](const double2* r, double2* z) { kgemv(ctx, dRedG, r, z, Nk, N, 1.0); };
      fr = fgmres(A64, M, dSb, x, cfg.stokes_rtol, cfg.stokes_restart, cfg.stokes_maxiter);
    }
    schur_matvec_fast(x, dSAx, false);
    vec_axpby(ctx, dSAx, make_double2(1.0, 0.0), dSb, make_double2(-1.0, 0.0), n);
    res = norm(dSAx) / std::max(norm(dSb), 1e-300);
    return true;
  }

  // counters of a BFBT solve and, when it failed, the rescue chain.  True
  // when a rescue changed x.
  bool bfbt_finish(const double2* th, double2* x, const FgmresResult& fr, double res) {
    ctr.n_bfbt_solves++;
    ctr.n_bfbt_iters += fr.iters;
    ctr.last_bfbt_true_res = res;
    ctr.last_K = 0;
    if (fr.info != 0 && !(res <= cfg.stokes_rtol) && !dense_feasible()) {
      // rescue without the dense route (its factor does not fit): rebuild the
      // BFBT blocks for the current eta and solve in FP64 with four times the
      // iteration budget; counted as a weak rescue
      ctr.n_bfbt_rescue++;
      bfbt_invalidate();
      bfbt_build();
      Op A64 = [&](const double2* v, double2* o) {
        if (fast) schur_matvec_fast(v, o, false);
        else schur_matvec(v, o);
      };
      Op M64 = [&](const double2* r, double2* z) {
        if (fast) kgemv(ctx, dRedG, r, z, Nk, N, 1.0);
        else lu_small_solve(ctx, dRedLU, dRedPiv, NN, r, z, N, Nk, 1.0, 1, nullptr);
      };
      FgmresResult f2 = fgmres(A64, M64, dSb, x, cfg.stokes_rtol, cfg.stokes_restart,
                               4 * cfg.stokes_maxiter);
      ctr.n_bfbt_iters += f2.iters;
      ctr.n_bfbt_rescue_weak++;
      res = schur_true_res(dSb, x);
      ctr.last_bfbt_true_res = res;
      return true;
    }
    if (fr.info != 0 && !(res <= cfg.stokes_rtol)) {
      // rescue chain (coupled_model.py:613-654)
      ctr.n_bfbt_rescue++;
      if (fast) lu_mode = 1;
      refresh();
      defect_solve(th, x);
      if (last_failed) {
        refresh();
        defect_solve(th, x);
        if (last_failed) ctr.n_defect_double_fail++;
      }
      res = schur_true_res(dSb, x);
      if (!(res <= cfg.stokes_rtol || !std::isfinite(res))) {
        if ((long long)Nk * N > 4096) ctr.n_bfbt_rescue_weak++;
        else {
          // the dense direct solve at this eta: the factor just refreshed
          // is exactly the LU of the assembled A(eta)
          lag_solve(dSb, x);
          ctr.n_bfbt_rescue_direct++;
        }
      }
      return true;
    }
    return false;
  }

  // deferred solves.  A Stokes solve launched inside cfl_dt (defer_stokes)
  // is completed after the CFL synchronisation; a temperature solve launched
  // inside a march (defer_theta) at the next synchronisation (the next dt
  // selection's memo test) or when any other entry point is called (settle)
  bool defer_stokes = false, defer_theta = false;
  const double2* stokes_pend_th = nullptr;
  double2* stokes_pend_x = nullptr;
  double2* theta_pend_out = nullptr;
  const double* theta_pend_gi = nullptr;
  bool theta_pend_sym = false;
  struct FlagScope {
    bool& f;
    explicit FlagScope(bool& f_, bool on = true) : f(f_) { f = on; }
    ~FlagScope() { f = false; }
  };

  // true when x changed after the deferred launch (an FP64 fallback or a
  // rescue): what was computed from it is stale
  bool stokes_finish() {
    double res = 0.0;
    FgmresResult fr = engine_result(0, &res);
    double2* x = stokes_pend_x;
    const double2* th = stokes_pend_th;
    stokes_pend_x = nullptr;
    stokes_pend_th = nullptr;
    bool changed = stokes_fp64_fallback(fr, res, x);
    changed = bfbt_finish(th, x, fr, res) || changed;
    return changed;
  }

  // counters of a temperature solve
  void theta_account(const FgmresResult& fr, double tr) {
    ctr.theta_last_res = tr;
    ctr.theta_last_iters = fr.iters;
    ctr.n_theta_iters += fr.iters;
    if (fr.info != 0) ctr.n_theta_nonconv++;
  }
  // non-finite values in the FP32 inner solves (info 3): the temperature
  // solve redone in FP64 with the step's operator and preconditioner
  void theta_fp64_redo(FgmresResult& fr, double& tr, const double* Gi) {
    ++n_fp64_fallback;
    Op A64 = [&](const double2* v, double2* o) { theta_matvec_fast(v, o, false); };
    Op M = [&](const double2* r, double2* z) { kgemv(ctx, Gi, r, z, Nk, N, -1.0); };
    fr = fgmres(A64, M, dKb, dRhs, cfg.theta_rtol, cfg.theta_restart, cfg.theta_maxiter);
    theta_matvec_fast(dRhs, sp[13], false);
    vec_axpby(ctx, sp[13], make_double2(1.0, 0.0), dKb, make_double2(-1.0, 0.0), n);
    tr = norm(sp[13]) / std::max(norm(dKb), 1e-300);
  }
  // true when the step's output changed after the deferred launch (the
  // FP64 redo); nothing between the launch and here touches the operator
  // state of that step (frozen velocity, BDF2 coefficients, rhs)
  bool theta_finish() {
    double tr = 0.0;
    FgmresResult fr = engine_result(1, &tr);
    double2* out = theta_pend_out;
    theta_pend_out = nullptr;
    bool redo = false;
    if (fr.info == 3) {
      theta_fp64_redo(fr, tr, theta_pend_gi);
      if (theta_pend_sym) project(dRhs, out);
      else vec_copy(ctx, out, dRhs, n);
      redo = true;
    }
    theta_account(fr, tr);
    return redo;
  }
  // completes deferred work before an entry point other than the march's
  // keep_prefetch: smc_step on the host input smc_production_dt just saw
  void settle(bool keep_prefetch = false) {
    if (!keep_prefetch) {
      mpf.valid = false;
      mpf_host.clear();
    }
    if (stokes_pend_x) {           // left by an exception inside cfl_dt
      eng_pending[0] = false;
      stokes_pend_x = nullptr;
    }
    if (theta_pend_out) theta_finish();
  }
  // the step's memo test, prefetched by cfl_dt inside a march: the values of
  // memo_compare for the step's projected temperature
  bool want_memo_prefetch = false;
  // the host input of the smc_production_dt call that made the prefetch
  // (smc_step on the same bytes uses it: the device copy is then identical)
  std::vector<unsigned char> mpf_host;
  struct MemoPrefetch {
    bool valid = false;
    const double2* src = nullptr;
    double v[3] = {0, 0, 0};
  } mpf;
  const double* memo_pre = nullptr;
  bool uses_memo() const { return cfg.model != SMC_MODEL_CONST && cfg.model != SMC_MODEL_ETA_Z; }
  // enqueues what step_theta(th) computes before its memo test: the mirror
  // projections (dTh1, dTh2), V th2 (sp[3]) and memo_compare into dScal[16..18]
  bool memo_prefetch_enqueue(const double2* th) {
    if (!uses_memo() || !memo_valid) return false;
    const double2* th2 = th;
    if (cfg.symmetrize != 0) {
      project(th, dTh1);
      project(dTh1, dTh2);
      th2 = dTh2;
    }
    zop(dV, 0, th2, sp[3]);
    memo_compare(ctx, th2, dMemoThat, sp[3], dMemoX, n, dScal + 16, dRed);
    return true;
  }

  void stokes_coupled(const double2* th, double2* psi, double2* om) {
    eta_of(th);
    SMC_CUDA(cudaMemcpyAsync(dLastEta, dEta, sizeof(double) * Nx * N, cudaMemcpyDeviceToDevice, stream));
    have_last_eta = true;
    eta_operator();
    if (cfg.precond == SMC_PRECOND_BFBT || fast) bfbt_solve(th, dSx);
    else legacy_solve(th, dSx);
    stokes_coupled_tail(psi, om);
  }
  void stokes_coupled_tail(double2* psi, double2* om) {
    zop(green_coupled(), NN, dSx, psi);
    // omega = -v (TALA: -v / rho_bar column by column, stokes_tala.py:327-340)
    if (tala) scale_cols(ctx, dSx, dRhoInv, -1.0, om, Nk, N);
    else vec_axpby(ctx, om, make_double2(-1.0, 0.0), dSx, make_double2(0.0, 0.0), n);
  }
  bool have_last_eta = false;

  // memoised Stokes solve of the coupled model (coupled_model.py:725-765)
  void stokes_memo(const double2* th, double2* psi, double2* om) {
    ProfScope psm(ctx, "stokes_memo_check");
    const double* pre = memo_pre;          // the test prefetched with the CFL reduction
    memo_pre = nullptr;
    if (!pre) zop(dV, 0, th, sp[3]);
    if (memo_valid) {
      double v[3];
      if (pre) {
        for (int q = 0; q < 3; ++q) v[q] = pre[q];
      } else {
        memo_compare(ctx, th, dMemoThat, sp[3], dMemoX, n, dScal, dRed);
        sync_read(dScal, 3);
        for (int q = 0; q < 3; ++q) v[q] = hbuf[q];
        if (theta_pend_out && theta_finish()) {
          // the temperature step that produced th was redone: test again
          zop(dV, 0, th, sp[3]);
          memo_compare(ctx, th, dMemoThat, sp[3], dMemoX, n, dScal, dRed);
          sync_read(dScal, 3);
          for (int q = 0; q < 3; ++q) v[q] = hbuf[q];
        }
      }
      bool eq = v[0] != 0.0;
      double den = std::max(v[2], 1e-300);
      if (eq || v[1] <= 1e-12 * den) {
        if (!eq) ctr.n_memo_hits++;
        vec_copy(ctx, psi, dMemoPsi, n);
        vec_copy(ctx, om, dMemoOm, n);
        return;
      }
    }
    stokes_coupled(th, dMemoPsi, dMemoOm);
    ctr.n_stokes++;
    vec_copy(ctx, dMemoThat, th, n);
    vec_copy(ctx, dMemoX, sp[3], n);
    memo_valid = true;
    vec_copy(ctx, psi, dMemoPsi, n);
    vec_copy(ctx, om, dMemoOm, n);
  }

  void stokes(const double2* th, double2* psi, double2* om) {
    if (cfg.model == SMC_MODEL_CONST) stokes_const(th, psi, om);
    else if (cfg.model == SMC_MODEL_ETA_Z) stokes_etaz(th, psi, om);
    else stokes_memo(th, psi, om);
  }

  // the two syntheses of a velocity (ux = VD psi, uz = V (-i k psi)) as one
  // two-job launch of each transform kernel (each job computes what its own
  // launch would)
  void synth_pair(const double2* psi, double* ux, double* uz, int Ng) {
    KFactor f; f.cre = 0.0; f.cim = -1.0; f.kpow = 1;       // -i k psi
    ZJob j[2];
    j[0].Z = dVD; j[0].X = psi; j[0].Y = sp[4];
    j[1].Z = dV; j[1].X = psi; j[1].Y = sp[9]; j[1].f = f;
    zmat_apply(ctx, j, 2, Nk, N, dkx);
    SynthJob s[2] = {{sp[4], ux}, {sp[9], uz}};
    synth_x(ctx, s, 2, Nk, N, Ng, Ng == Np ? dtwNp : dtwNx);
  }
  void velocity(const double2* psi, double* ux, double* uz) {
    synth_pair(psi, ux, uz, Nx);
    if (tala) grid_div_rho(ctx, ux, uz, dRho, (long long)Nx * N, N);   // u = curl(Psi) / rho_bar
  }

  double cfl_dt(const double2* th, double safety, double dtmax, double dtmin) {
    mpf.valid = false;
    if (theta_pend_out && !uses_memo()) settle();
    {
      FlagScope fs(defer_stokes);
      stokes(th, dPsi, dOm);
    }
    ProfScope ps(ctx, "cfl_velocity");
    velocity(dPsi, gr[0], gr[1]);
    reduce_maxabs2(ctx, gr[0], gr[1], (long long)Nx * N, dScal, dRed);
    const bool pre = want_memo_prefetch && memo_prefetch_enqueue(th);
    sync_read(dScal, pre ? 19 : 1);
    double vmax = hbuf[0];
    if (pre) {
      mpf.valid = true;
      mpf.src = th;
      for (int q = 0; q < 3; ++q) mpf.v[q] = hbuf[16 + q];
    }
    if (stokes_pend_x && stokes_finish()) {
      // the solve's x changed after its launch: psi, omega and the velocity again
      stokes_coupled_tail(dMemoPsi, dMemoOm);
      vec_copy(ctx, dPsi, dMemoPsi, n);
      vec_copy(ctx, dOm, dMemoOm, n);
      velocity(dPsi, gr[0], gr[1]);
      reduce_maxabs2(ctx, gr[0], gr[1], (long long)Nx * N, dScal, dRed);
      sync_read(dScal, 1);
      vmax = hbuf[0];
    }
    if (!(vmax >= 1e-12)) vmax = (vmax != vmax) ? vmax : 1e-12;
    double dt = safety * std::min(cfg.Lx / Nx, dzmin) / vmax;
    return std::min(std::max(dt, dtmin), dtmax);
  }

  double production_dt(const double2* th, double safety, double dtmax) {
    double fac = std::min(std::max(safety, 0.0), 80.0);
    return std::min(dtmax, cfl_dt(th, fac, dtmax, 1e-10));
  }

  void project(const double2* in, double2* out) {
    zop(dV, 0, in, sp[5]);
    zop(dVi, 0, sp[5], out, KFactor(), 1);
  }

  // ------------------------------------------------------- Phi source
  // (Di/Ra) F(Phi) with tau rows zeroed, from psi* and the step's eta
  // (physics/dissipation.py:313-378, :445-459)
  void phi_grid(const double2* psi, const double* eta_pad, double coef, double* out, int accumulate) {
    KFactor fik; fik.cre = 0.0; fik.cim = 1.0; fik.kpow = 1;
    synth(psi, dVD, fik, gr[6], Np, sp[6]);                 // exx = i k D psi
    KFactor h; h.cre = 0.5;
    KFactor hk; hk.cre = 0.5; hk.kpow = 2;
    zop(dVD2, 0, psi, sp[7], h);                             // V (exz) = 0.5 (V D2 psi + k^2 V psi)
    zop(dV, 0, psi, sp[7], hk, 0, 1);
    SynthJob s{sp[7], gr[7]};
    synth_x(ctx, &s, 1, Nk, N, Np, dtwNp);
    // ezz = -exx and tr = 0 exactly, so gzz^2 = gxx^2 and gtr = 0
    grid_phi(ctx, gr[6], gr[6], gr[7], nullptr, eta_pad, coef, out, (long long)Np * N, accumulate);
  }

  void phi_source(const double2* psi, double2* out) {
    const double* ep = nullptr;
    if (cfg.model == SMC_MODEL_ETA_Z) ep = dEtaPadZ;
    else if (cfg.model == SMC_MODEL_ETA_T) {
      if (have_last_eta) { eta_pad_from_grid(dLastEta, gr[8]); ep = gr[8]; }
      else ep = dEtaPadZ;
    }
    phi_grid(psi, ep, 1.0, gr[9], 0);
    KFactor f; f.cre = cfg.dissipation_number / cfg.Ra;
    analyze(gr[9], Np, out, sp[8], f, 1);
  }

  // -------------------------------------------------------- const step
  void step_const(const double2* th, double2* out, double dt) {
    stokes_const(th, dPsi, dOm);
    ZJob jobs[4];
    KFactor ik; ik.cre = 0.0; ik.cim = 1.0; ik.kpow = 1;
    KFactor mik; mik.cre = 0.0; mik.cim = -1.0; mik.kpow = 1;
    jobs[0].Z = dV; jobs[0].X = th; jobs[0].Y = sp[0]; jobs[0].f = ik;     // thx
    jobs[1].Z = dVD; jobs[1].X = th; jobs[1].Y = sp[1];                   // thz
    jobs[2].Z = dVD; jobs[2].X = dPsi; jobs[2].Y = sp[2];                 // ux
    jobs[3].Z = dV; jobs[3].X = dPsi; jobs[3].Y = sp[3]; jobs[3].f = mik; // uz
    zmat_apply(ctx, jobs, 4, Nk, N, dkx);
    SynthJob sj[4] = {{sp[0], gr[0]}, {sp[1], gr[1]}, {sp[2], gr[2]}, {sp[3], gr[3]}};
    synth_x(ctx, sj, 4, Nk, N, Np, dtwNp);
    grid_explicit_nonlinear(ctx, gr[2], gr[3], gr[0], gr[1], cfg.internal_heating, gr[4],
                            (long long)Np * N);
    if (cfg.dissipation_number != 0.0)
      phi_grid(dPsi, nullptr, cfg.dissipation_number / cfg.Ra, gr[4], 1);
    analyze(gr[4], Np, sp[5], sp[6]);                                      // Nc
    const_rhs(ctx, th, sp[5], dt, sp[7], n);
    LamSlot& L = lam_lu(1.0 / dt);
    lu_small_solve(ctx, L.LU, L.piv, NN, sp[7], out, N, Nk, -1.0, 1, nullptr);
    ctr.n_steps++;
  }

  // ---------------------------------------------- implicit theta step
  void theta_matvec(const double2* v, double2* out) {
    ProfScope ps(ctx, "theta_matvec");
    ZJob jobs[2];
    KFactor ik; ik.cre = 0.0; ik.cim = 1.0; ik.kpow = 1;
    jobs[0].Z = dV; jobs[0].X = v; jobs[0].Y = sp[9]; jobs[0].f = ik;
    jobs[1].Z = dVD; jobs[1].X = v; jobs[1].Y = sp[10];
    zmat_apply(ctx, jobs, 2, Nk, N, dkx);
    SynthJob sj[2] = {{sp[9], gr[2]}, {sp[10], gr[3]}};
    synth_x(ctx, sj, 2, Nk, N, Np, dtwNp);
    grid_advect_product(ctx, gr[0], gr[1], gr[2], gr[3], gr[4], (long long)Np * N);
    AnaJob a{gr[4], sp[11]};
    analysis_x(ctx, &a, 1, Nk, N, Np, dtwNp, 1.0 / Np);
    if (tala) tala_theta_combine(ctx, v, sp[11], dMrho, dMrhoVi, dD2, dV, dkx, a0, out, Nk, N);
    else theta_combine(ctx, v, sp[11], dD2, dVi, dV, dkx, a0, out, Nk, N);
  }

  void set_step(double dt, bool have_p, double dtp) {
    if (!have_p) {
      a0 = b0 = 1.0 / dt;
      b1 = 0.0;
      ctr.n_be_fallback++;
      return;
    }
    double r = dt / dtp;
    a0 = (1.0 + 2.0 * r) / ((1.0 + r) * dt);
    b0 = (1.0 + r) / dt;
    b1 = r * r / ((1.0 + r) * dt);
  }

  void step_theta(const double2* th_in, double2* out, double dt) {
    // a deferred solve of the step before (smc_march: no dt selection in
    // between) is completed before th_in is read
    if (theta_pend_out) theta_finish();
    const bool sym = cfg.symmetrize != 0;
    // the projections and the memo test prefetched by cfl_dt for this state
    const bool pre = mpf.valid && mpf.src == th_in;
    mpf.valid = false;
    const double2* th1 = th_in;
    const double2* th2 = th_in;
    if (sym) {
      if (!pre) {
        project(th_in, dTh1);
        project(dTh1, dTh2);
      }
      th1 = dTh1;
      th2 = dTh2;
    }
    if (pre) memo_pre = mpf.v;
    stokes(th2, dPsi, dOm);
    memo_pre = nullptr;
    vec_copy(ctx, dPsiN, dPsi, n);
    const double2* ps = dPsi;
    if (have_prev) { extrapolate(ctx, dPsi, dPsiPrev, dPsiStar, n); ps = dPsiStar; }
    // frozen velocity on the padded grid
    {
      ProfScope psa(ctx, "theta_rhs");
      synth_pair(ps, gr[0], gr[1], Np);
    }
    const double2* phi = nullptr;
    if (cfg.dissipation_number != 0.0) { phi_source(ps, dPhi); phi = dPhi; }
    set_step(dt, have_prev, dt_prev);
    {
      ProfScope psa(ctx, "theta_rhs");
      if (tala) {
        // adiabatic source rho_bar u_z [1 - Di (1 - z + theta)] on the padded
        // grid, truncated back with its tau rows zeroed (implicit_theta.py:336-350)
        synth(th2, dV, KFactor(), dTalaThG, Np, sp[12]);
        tala_adiabatic_grid(ctx, gr[1], dTalaThG, dRho, dz, cfg.dissipation_number, dTalaAdG,
                            (long long)Np * N, N);
        analyze(dTalaAdG, Np, dTalaAd, sp[12], KFactor(), 1);
        tala_theta_rhs(ctx, th2, dPrev, dMrho, dRhoC, dTalaAd, phi, b0, b1, cfg.internal_heating,
                       dKb, Nk, N);
      } else {
        theta_rhs(ctx, th2, dPrev, ps, phi, dkx, b0, b1, cfg.internal_heating, dKb, Nk, N);
      }
    }
    Op A = [&](const double2* v, double2* o) { theta_matvec(v, o); };
    LamSlot* Lp = &lam_lu(a0);
    double* LU = Lp->LU;
    int* piv = Lp->piv;
    double* Gi = Lp->Ginv;
    Op M = [&](const double2* r, double2* z) {
      ProfScope ps(ctx, "theta_precond");
      if (fast) {
        kgemv(ctx, Gi, r, z, Nk, N, -1.0);   // -(A^{-1} P) r
      } else {
        lu_small_solve(ctx, LU, piv, NN, r, z, N, Nk, -1.0, 1, nullptr);
      }
    };
    FgmresResult fr;
    bool deferred = false;
    if (fast) {
      to_float(ctx, gr[0], dUx32, (long long)Np * N);
      to_float(ctx, gr[1], dUz32, (long long)Np * N);
      Op A64 = [&](const double2* v, double2* o) { theta_matvec_fast(v, o, false); };
      Op A32 = [&](const double2* v, double2* o) { theta_matvec_fast(v, o, true); };
      double tr = 0.0;
      if (inner_fp32) {
        if (use_engine) {
          // guess: the last step's temperature extrapolated linearly in time
          if (warm_start && (warm_extrap & 2) && have_prev && dt_prev > 0.0) {
            const double r = dt / dt_prev;
            vec_axpby(ctx, dRhs, make_double2(-r, 0.0), dPrev, make_double2(1.0 + r, 0.0), n);
          }
          // inside a march the result is read at the next dt selection's
          // memo test: the host enqueues the rest of the step meanwhile
          deferred = defer_theta && uses_memo() && memo_valid && !batch_mode &&
                     !(eng_phase && prof.enabled);
          fr = engine_refine(1, dKb, dRhs, cfg.theta_rtol, cfg.theta_maxiter, cfg.theta_restart,
                             Lp->GinvT32, Lp->GinvT64, -1.0, &tr, deferred);
          if (deferred) {
            theta_pend_out = out;
            theta_pend_gi = Gi;
            theta_pend_sym = sym;
          }
        } else {
          InnerSolve inner = [&](const double2* r, double2* e, double tol, int mi) {
            return fgmres(A32, M, r, e, tol, cfg.theta_restart, mi);
          };
          fr = fgmres_refined(A64, inner, dKb, dRhs, cfg.theta_rtol, cfg.theta_maxiter, inner_floor[1],
                              &tr);
        }
        if (!deferred && fr.info == 3) theta_fp64_redo(fr, tr, Gi);
      } else {
        if (use_engine)
          fr = engine_solve(1, false, dKb, dRhs, cfg.theta_rtol, cfg.theta_restart,
                            cfg.theta_maxiter, Lp->GinvT64, -1.0);
        else
          fr = fgmres(A64, M, dKb, dRhs, cfg.theta_rtol, cfg.theta_restart, cfg.theta_maxiter);
        theta_matvec_fast(dRhs, sp[13], false);
        vec_axpby(ctx, sp[13], make_double2(1.0, 0.0), dKb, make_double2(-1.0, 0.0), n);
        tr = norm(sp[13]) / std::max(norm(dKb), 1e-300);
      }
      if (!deferred) theta_account(fr, tr);
    } else {
      fr = fgmres(A, M, dKb, dRhs, cfg.theta_rtol, cfg.theta_restart, cfg.theta_maxiter);
      // true relative residual of the accepted solution (implicit_theta.py:510-516)
      theta_matvec(dRhs, sp[13]);
      vec_axpby(ctx, sp[13], make_double2(1.0, 0.0), dKb, make_double2(-1.0, 0.0), n);
      double bn = std::max(norm(dKb), 1e-300);
      theta_account(fr, norm(sp[13]) / bn);
    }
    ctr.n_theta_solves++;
    ctr.n_steps++;
    if (sym) project(dRhs, out);
    else vec_copy(ctx, out, dRhs, n);
    vec_copy(ctx, dPrev, th1, n);
    vec_copy(ctx, dPsiPrev, dPsiN, n);
    dt_prev = dt;
    have_prev = true;
  }

  void step(const double2* in, double2* out, double dt) {
    if (cfg.model == SMC_MODEL_CONST) step_const(in, out, dt);
    else step_theta(in, out, dt);
    ++steps_done;
    step_dt[1] = step_dt[0];
    step_dt[0] = dt;
  }

  // -------------------------------------------------------------- FGMRES
  // right-preconditioned, zero initial guess (core/krylov_fgmres.py:60-179)
  FgmresResult fgmres(const Op& A, const Op& M, const double2* b, double2* x, double rtol,
                      int restart, int maxiter) {
    FgmresResult res;
    const int m = std::max(1, std::min(restart, mmax));
    vec_zero(ctx, x, n * sizeof(double2));
    double beta = norm(b);                 // r0 = b - A(0) = b
    const double tol = rtol * beta;
    if (beta <= tol) { res.info = 0; res.iters = 0; return res; }
    vec_copy(ctx, dKr, b, n);
    int total = 0, info = 1;
    std::vector<cplx> H((size_t)(m + 1) * m), g(m + 1), sn(m);
    std::vector<double> cs(m);
    std::vector<double2> hv(m + 2);
    auto Hij = [&](int i, int j) -> cplx& { return H[(size_t)i * m + j]; };
    while (total < maxiter) {
      std::fill(H.begin(), H.end(), cplx(0, 0));
      std::fill(g.begin(), g.end(), cplx(0, 0));
      vec_div(ctx, dKr, beta, dKV, n);
      g[0] = beta;
      int k = 0;
      for (int j = 0; j < m; ++j) {
        if (total >= maxiter) { info = 1; break; }
        double2* Vj = dKV + (size_t)j * n;
        double2* Zj = dKZ + (size_t)j * n;
        M(Vj, Zj);
        A(Zj, dKw);
        if (fast) {
          ProfScope ps(ctx, "fgmres_cgs2");
          cgs2(ctx, dKV, j, n, dKw, dKh, dCgsPart);
        } else {
          ProfScope ps(ctx, "fgmres_mgs");
          mgs(ctx, dKV, j, n, dKw, dKh);
        }
        SMC_CUDA(cudaMemcpyAsync(hv.data(), dKh, (j + 2) * sizeof(double2), cudaMemcpyDeviceToHost, stream));
        SMC_CUDA(cudaStreamSynchronize(stream));
        for (int i = 0; i <= j; ++i) Hij(i, j) = cplx(hv[i].x, hv[i].y);
        const double hn = hv[j + 1].x;
        Hij(j + 1, j) = hn;
        for (int i = 0; i < j; ++i) {
          cplx t = cs[i] * Hij(i, j) + sn[i] * Hij(i + 1, j);
          Hij(i + 1, j) = -std::conj(sn[i]) * Hij(i, j) + cs[i] * Hij(i + 1, j);
          Hij(i, j) = t;
        }
        // complex Givens (krylov_fgmres.py:42-57)
        cplx a = Hij(j, j), bb = Hij(j + 1, j);
        double aa = std::abs(a), bba = std::abs(bb);
        double c;
        cplx s, rjj;
        if (bba == 0.0) { c = 1.0; s = 0.0; rjj = a; }
        else if (aa == 0.0) { c = 0.0; s = std::conj(bb) / bba; rjj = bba; }
        else {
          double den = std::sqrt(aa * aa + bba * bba);
          c = aa / den;
          s = c * std::conj(bb) / std::conj(a);
          rjj = c * (aa * aa + bba * bba) / std::conj(a);
        }
        cs[j] = c; sn[j] = s;
        Hij(j, j) = rjj;
        Hij(j + 1, j) = 0.0;
        cplx t = c * g[j] + s * g[j + 1];
        g[j + 1] = -std::conj(s) * g[j] + c * g[j + 1];
        g[j] = t;
        ++total;
        k = j + 1;
        if (std::abs(g[j + 1]) <= tol) { info = 0; break; }
        if (hn == 0.0) { info = 2; break; }
        vec_div(ctx, dKw, hn, dKV + (size_t)(j + 1) * n, n);
      }
      if (k == 0) break;
      // back substitution of the triangular H[:k,:k] y = g[:k]
      std::vector<cplx> y(k);
      for (int i = k - 1; i >= 0; --i) {
        cplx s = g[i];
        for (int q = i + 1; q < k; ++q) s -= Hij(i, q) * y[q];
        y[i] = s / Hij(i, i);
      }
      std::vector<double2> yd(k);
      for (int i = 0; i < k; ++i) yd[i] = make_double2(y[i].real(), y[i].imag());
      SMC_CUDA(cudaMemcpyAsync(dKy, yd.data(), k * sizeof(double2), cudaMemcpyHostToDevice, stream));
      krylov_update(ctx, x, dKZ, dKy, k, n);
      if (info == 0 || info == 2) break;
      A(x, dKr);
      vec_axpby(ctx, dKr, make_double2(1.0, 0.0), b, make_double2(-1.0, 0.0), n);   // r = b - Ax
      beta = norm(dKr);
      if (beta <= tol) { info = 0; break; }
    }
    res.info = info;
    res.iters = total;
    return res;
  }

  ~Model() {
    if (stream) { cudaStreamSynchronize(stream); cudaStreamDestroy(stream); }
    if (hbuf) cudaFreeHost(hbuf);
    if (hpin) cudaFreeHost(hpin);
    if (hBatchRes) cudaFreeHost((void*)hBatchRes);
    if (batch_ready) cudaEventDestroy(batch_ready);
    for (auto e : eng_done)
      if (e) cudaEventDestroy(e);
    if (bfbt_exec) cudaGraphExecDestroy(bfbt_exec);
    if (bfbt_graph) cudaGraphDestroy(bfbt_graph);
  }
};

// small helper kernels of the runtime
__global__ void smc_realpart_kernel(const double2* in, double* out, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[i].x;
}
__global__ void smc_comm_kernel(const double* a, const double* b, const double* c, double* out,
                                long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (a[i] - 2.0 * b[i]) + c[i];
}
void Model::realpart(const double2* in, double* out, int count) {
  smc_realpart_kernel<<<ceil_div(count, 128), 128, 0, stream>>>(in, out, count);
  SMC_LAUNCH_CHECK(ctx);
}
void Model::comm_combine(const double* a, const double* b, const double* c, double* out,
                         long long cnt) {
  smc_comm_kernel<<<ceil_div(cnt, 256), 256, 0, stream>>>(a, b, c, out, cnt);
  SMC_LAUNCH_CHECK(ctx);
}

}  // namespace smc

// ====================================================================== C ABI
struct smc_handle {
  smc::Model m;
};

using smc::Model;

namespace {

int fail(const std::exception& e) {
  smc::g_last_error = e.what();
  return -1;
}

void copy_in(Model& m, double2* dst, const double* src, int mem, long long count) {
  auto kind = mem == SMC_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  SMC_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(double2), kind, m.stream));
}
void copy_out(Model& m, double* dst, const void* src, int mem, long long bytes) {
  auto kind = mem == SMC_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  SMC_CUDA(cudaMemcpyAsync(dst, src, bytes, kind, m.stream));
  SMC_CUDA(cudaStreamSynchronize(m.stream));
}

void validate(const smc_config* c) {
  if (!c) throw std::runtime_error("null config");
  if (c->abi_version != SMC_ABI_VERSION) throw std::runtime_error("smc_config.abi_version mismatch");
  if (c->model < 0 || c->model > 2) throw std::runtime_error("unknown model");
  if (c->Nx < 4 || c->Nz < 4) throw std::runtime_error("Nx, Nz must be >= 4");
  if (c->Nx % 2) throw std::runtime_error("Nx must be even");
  if (!(c->Ra > 0) || !(c->Lx > 0) || !(c->deta_T > 0)) throw std::runtime_error("Ra, Lx, deta_T must be positive");
  if (!(c->eta_min > 0) || !(c->eta_max > c->eta_min)) throw std::runtime_error("bad eta window");
  if (c->lag < 1 || c->max_K < 1 || c->K < 0) throw std::runtime_error("bad defect-correction settings");
  if (c->theta_restart < 1 || c->stokes_restart < 1) throw std::runtime_error("bad restart");
  if (c->precision != SMC_FP64 && c->precision != SMC_MIXED) throw std::runtime_error("unknown precision");
  if (!std::isfinite(c->arrhenius_V) || c->arrhenius_V < 0.0)
    throw std::runtime_error("arrhenius_V must be finite and >= 0");
  if (c->arrhenius_V > 0.0 &&
      (c->model != SMC_MODEL_ETA_T || !(c->arrhenius_Ts > 0.0) || !std::isfinite(c->arrhenius_E)))
    throw std::runtime_error("arrhenius_V > 0 (pV law) needs model ETA_T, arrhenius_Ts > 0 and a finite "
                             "calibrated arrhenius_E");
  if (c->compressibility != SMC_BOUSSINESQ && c->compressibility != SMC_TALA)
    throw std::runtime_error("unknown compressibility");
  if (c->compressibility == SMC_TALA) {
    if (!std::isfinite(c->dissipation_number) || c->dissipation_number < 0.0)
      throw std::runtime_error("compressibility TALA needs a finite dissipation_number >= 0");
    if (c->precision != SMC_FP64)
      throw std::runtime_error("compressibility TALA runs the FP64 form only (precision SMC_FP64)");
    if (c->model == SMC_MODEL_ETA_T && c->precond != SMC_PRECOND_LEGACY)
      throw std::runtime_error("compressibility TALA with precond BFBT: the spectral BFBT model is "
                               "Boussinesq-only; use SMC_PRECOND_LEGACY (config.py:462-470)");
  }
}

}  // namespace

extern "C" {

void smc_config_defaults(smc_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->abi_version = SMC_ABI_VERSION;
  c->model = SMC_MODEL_ETA_T;
  c->Nx = 64; c->Nz = 96;
  c->Ra = 1e4; c->Lx = 2.0; c->deta_T = 1000.0;
  c->eta_min = 1e-3; c->eta_max = 1e3;
  c->precond = SMC_PRECOND_LEGACY;
  c->symmetrize = 1;
  c->lag = 16; c->K = 3; c->max_K = 8;
  c->defect_tol = 1e-8;
  c->eta_drift_tol = 0.1;
  c->stokes_rtol = 1e-8; c->theta_rtol = 1e-10;
  c->theta_maxiter = 200; c->theta_restart = 40;
  c->stokes_restart = 80; c->stokes_maxiter = 800;
  c->precision = SMC_FP64;
  c->device = 0;
}

int smc_create(const smc_config* cfg, smc_handle** out) {
  try {
    validate(cfg);
    std::unique_ptr<smc_handle> h(new smc_handle());
    h->m.cfg = *cfg;
    h->m.setup();
    *out = h.release();
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

int smc_destroy(smc_handle* h) {
  delete h;
  return 0;
}

// every entry point but smc_advance first completes the deferred work of
// the handle's last march (settle)
#define SMC_GUARD_IMPL(h, settle_first, ...)                 \
  try {                                                      \
    if (!(h)) throw std::runtime_error("null handle");       \
    SMC_CUDA(cudaSetDevice((h)->m.device));                  \
    if (settle_first) (h)->m.settle();                       \
    __VA_ARGS__;                                             \
    return 0;                                                \
  } catch (const std::exception& e) {                        \
    return fail(e);                                          \
  }
#define SMC_GUARD(h, ...) SMC_GUARD_IMPL(h, true, __VA_ARGS__)

int smc_step(smc_handle* h, const double* in, double* out, int mem, double dt) {
  SMC_GUARD_IMPL(h, false, {
    Model& m = h->m;
    // the input smc_production_dt just took: its prefetched projections and
    // memo test hold for it (bytes compared on the host)
    const bool same = mem == SMC_HOST && !m.mpf_host.empty() &&
                      m.mpf_host.size() == (size_t)m.n * sizeof(double2) &&
                      std::memcmp(m.mpf_host.data(), in, m.mpf_host.size()) == 0;
    m.settle(same);
    m.mpf_host.clear();
    smc::BatchScope bs(m.device, m.batch_mode);
    copy_in(m, m.dIn, in, mem, m.n);
    {
      // the temperature solve's result is read with the copy of the output
      Model::FlagScope df(m.defer_theta);
      m.step(m.dIn, m.dOut, dt);
    }
    copy_out(m, out, m.dOut, mem, m.n * sizeof(double2));
    if (m.theta_pend_out && m.theta_finish()) copy_out(m, out, m.dOut, mem, m.n * sizeof(double2));
    m.check_tc();
  })
}

int smc_cfl_dt(smc_handle* h, const double* in, int mem, double safety, double dtmax, double dtmin,
               double* dt_out) {
  SMC_GUARD(h, {
    Model& m = h->m;
    smc::BatchScope bs(m.device, m.batch_mode);
    copy_in(m, m.dIn, in, mem, m.n);
    *dt_out = m.cfl_dt(m.dIn, safety, dtmax, dtmin);
  })
}

int smc_production_dt(smc_handle* h, const double* in, int mem, double safety, double dtmax,
                      double* dt_out) {
  SMC_GUARD(h, {
    Model& m = h->m;
    smc::BatchScope bs(m.device, m.batch_mode);
    copy_in(m, m.dIn, in, mem, m.n);
    {
      // prefetch the step's projections and memo test too (host input: a
      // following smc_step on the same bytes uses them, as a march does)
      Model::FlagScope pf(m.want_memo_prefetch, mem == SMC_HOST);
      *dt_out = m.production_dt(m.dIn, safety, dtmax);
    }
    if (mem == SMC_HOST && m.mpf.valid) {
      const unsigned char* p = reinterpret_cast<const unsigned char*>(in);
      m.mpf_host.assign(p, p + m.n * sizeof(double2));
    }
  })
}

int smc_march_adaptive(smc_handle* h, const double* in, double* out, int mem, double tstop,
                       double safety, double dtmax, long long max_steps, smc_march_info* info) {
  SMC_GUARD(h, {
    Model& m = h->m;
    smc::BatchScope bs(m.device, m.batch_mode);
    copy_in(m, m.dS0, in, mem, m.n);
    double2* cur = m.dS0;
    double2* nxt = m.dS1;
    double t = 0.0, dt = NAN;
    long long steps = 0;
    while (t < tstop && (max_steps <= 0 || steps < max_steps)) {
      {
        Model::FlagScope pf(m.want_memo_prefetch);
        dt = m.production_dt(cur, safety, dtmax);
      }
      {
        Model::FlagScope df(m.defer_theta);
        m.step(cur, nxt, dt);
      }
      std::swap(cur, nxt);
      t += dt;
      ++steps;
    }
    m.settle();
    copy_out(m, out, cur, mem, m.n * sizeof(double2));
    m.check_tc();
    if (info) { info->steps = steps; info->t = t; info->dt = dt; }
  })
}

int smc_set_state(smc_handle* h, const double* that, int mem) {
  SMC_GUARD(h, {
    Model& m = h->m;
    copy_in(m, m.dS0, that, mem, m.n);
    SMC_CUDA(cudaStreamSynchronize(m.stream));
    m.resident_cur0 = true;
    m.t_resident = 0.0;
  })
}

int smc_get_state(smc_handle* h, double* out, int mem) {
  SMC_GUARD(h, {
    Model& m = h->m;
    copy_out(m, out, m.resident_cur0 ? m.dS0 : m.dS1, mem, m.n * sizeof(double2));
  })
}

namespace smc {
// CFL-limited steps of the resident state until t >= tstop or max_steps
// (the loop of api.march_adaptive, api.py:179-189)
void advance_resident(Model& m, double tstop, long long max_steps, double safety, double dtmax,
                      smc_march_info* info) {
    double2* cur = m.resident_cur0 ? m.dS0 : m.dS1;
    double2* nxt = m.resident_cur0 ? m.dS1 : m.dS0;
    double dt = NAN;
    long long steps = 0;
    while (m.t_resident < tstop && (max_steps <= 0 || steps < max_steps)) {
      // the step's projections and memo test travel with the CFL
      // reduction, and the temperature solve's result is read at the next
      // memo test: two synchronisations per step
      {
        smc::ProfScope ps(m.ctx, "step.dt_select");
        Model::FlagScope pf(m.want_memo_prefetch);
        dt = m.production_dt(cur, safety, dtmax);
      }
      {
        smc::ProfScope ps(m.ctx, "step.advance");
        Model::FlagScope df(m.defer_theta);
        m.step(cur, nxt, dt);
      }
      std::swap(cur, nxt);
      m.resident_cur0 = !m.resident_cur0;
      m.t_resident += dt;
      ++steps;
    }
    if (info) { info->steps = steps; info->t = m.t_resident; info->dt = dt; }
}
}  // namespace smc

int smc_advance(smc_handle* h, double tstop, long long max_steps, double safety, double dtmax,
                smc_march_info* info) {
  SMC_GUARD_IMPL(h, false, {
    Model& m = h->m;
    smc::BatchScope bs(m.device, m.batch_mode);
    smc::advance_resident(m, tstop, max_steps, safety, dtmax, info);
    m.check_tc();
  })
}

int smc_profile(smc_handle* h, int enable) {
  SMC_GUARD(h, {
    if (enable < 0 || enable > 2) throw std::runtime_error("smc_profile: enable must be 0, 1 or 2");
    h->m.prof.reset();
    h->m.prof.enabled = enable != 0;
    h->m.prof.engine_only = enable == 2;
  })
}

int smc_profile_get(smc_handle* h, int slot, const char** name, double* ms, long long* launches,
                    double* work, int* work_is_bytes) {
  SMC_GUARD(h, {
    smc::Profiler& p = h->m.prof;
    p.resolve();
    if (slot < 0 || slot >= smc::Profiler::MAXTAG || p.names[slot] == nullptr) {
      *name = nullptr;
    } else {
      *name = p.names[slot];
      *ms = p.ms[slot];
      *launches = p.launches[slot];
      *work = p.work[slot];
      *work_is_bytes = p.work_is_bytes[slot];
    }
  })
}

int smc_march(smc_handle* h, const double* in, double* out, int mem, double dt, long long nsteps) {
  SMC_GUARD(h, {
    Model& m = h->m;
    smc::BatchScope bs(m.device, m.batch_mode);
    copy_in(m, m.dS0, in, mem, m.n);
    double2* cur = m.dS0;
    double2* nxt = m.dS1;
    for (long long s = 0; s < nsteps; ++s) {
      Model::FlagScope df(m.defer_theta);     // read at the next step's memo test
      m.step(cur, nxt, dt);
      std::swap(cur, nxt);
    }
    m.settle();
    copy_out(m, out, cur, mem, m.n * sizeof(double2));
    m.check_tc();
  })
}

int smc_diagnostics(smc_handle* h, const double* in, int mem, smc_diag* out) {
  SMC_GUARD(h, {
    Model& m = h->m;
    copy_in(m, m.dIn, in, mem, m.n);
    m.stokes(m.dIn, m.dPsi, m.dOm);
    m.velocity(m.dPsi, m.gr[0], m.gr[1]);
    m.synth(m.dIn, m.dV, smc::KFactor(), m.gr[2], m.Nx, m.sp[4]);
    smc::diagnostics_reduce(m.ctx, m.gr[0], m.gr[1], m.gr[2], m.dIn, m.dD, m.dV, m.dwq, m.Nx, m.N, m.dScal,
                            m.dRed, m.dDiagTicket);
    m.sync_read(m.dScal, 6);
    out->Nu_top = m.hbuf[0]; out->Nu_bot = m.hbuf[1]; out->Nu_energy = m.hbuf[2];
    out->urms = m.hbuf[3]; out->umax = m.hbuf[4]; out->amp = m.hbuf[5];
  })
}

int smc_stokes(smc_handle* h, const double* in, int mem, double* psi_out, double* om_out) {
  SMC_GUARD(h, {
    Model& m = h->m;
    copy_in(m, m.dIn, in, mem, m.n);
    m.stokes(m.dIn, m.dPsi, m.dOm);
    copy_out(m, psi_out, m.dPsi, mem, m.n * sizeof(double2));
    copy_out(m, om_out, m.dOm, mem, m.n * sizeof(double2));
  })
}

int smc_velocity(smc_handle* h, const double* psi, int mem, double* ux, double* uz) {
  SMC_GUARD(h, {
    Model& m = h->m;
    copy_in(m, m.dIn, psi, mem, m.n);
    m.velocity(m.dIn, m.gr[0], m.gr[1]);
    copy_out(m, ux, m.gr[0], mem, sizeof(double) * m.Nx * m.N);
    copy_out(m, uz, m.gr[1], mem, sizeof(double) * m.Nx * m.N);
  })
}

int smc_project_mirror(smc_handle* h, const double* in, double* out, int mem) {
  SMC_GUARD(h, {
    Model& m = h->m;
    copy_in(m, m.dIn, in, mem, m.n);
    m.project(m.dIn, m.dOut);
    copy_out(m, out, m.dOut, mem, m.n * sizeof(double2));
  })
}

int smc_transform(smc_handle* h, int kind, const double* in, double* out, int mem) {
  SMC_GUARD(h, {
    Model& m = h->m;
    long long gN = (long long)m.Nx * m.N, gP = (long long)m.Np * m.N;
    auto kin = mem == SMC_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (kind == SMC_GRID || kind == SMC_SYNTH_PAD) {
      copy_in(m, m.dIn, in, mem, m.n);
      int Ng = kind == SMC_GRID ? m.Nx : m.Np;
      m.synth(m.dIn, m.dV, smc::KFactor(), m.gr[0], Ng, m.sp[0]);
      copy_out(m, out, m.gr[0], mem, sizeof(double) * Ng * m.N);
    } else if (kind == SMC_COEFFS) {
      SMC_CUDA(cudaMemcpyAsync(m.gr[0], in, sizeof(double) * gN, kin, m.stream));
      m.analyze(m.gr[0], m.Nx, m.dOut, m.sp[0]);
      copy_out(m, out, m.dOut, mem, m.n * sizeof(double2));
    } else if (kind == SMC_TRUNC_PAD) {
      SMC_CUDA(cudaMemcpyAsync(m.gr[0], in, sizeof(double) * gP, kin, m.stream));
      smc::AnaJob a{m.gr[0], m.dOut};
      smc::analysis_x(m.ctx, &a, 1, m.Nk, m.N, m.Np, m.dtwNp, 1.0 / m.Np);
      copy_out(m, out, m.dOut, mem, m.n * sizeof(double2));
    } else {
      throw std::runtime_error("unknown transform kind");
    }
    m.check_tc();
  })
}

int smc_eta_of(smc_handle* h, const double* in, int mem, double* eta_out) {
  SMC_GUARD(h, {
    Model& m = h->m;
    if (m.cfg.model != SMC_MODEL_ETA_T) throw std::runtime_error("eta_of needs the eta_T model");
    copy_in(m, m.dIn, in, mem, m.n);
    m.eta_of(m.dIn);
    copy_out(m, eta_out, m.dEta, mem, sizeof(double) * m.Nx * m.N);
  })
}

int smc_dissipation_eta(smc_handle* h, double* eta_out, int mem, int* rows_out) {
  SMC_GUARD(h, {
    Model& m = h->m;
    if (!rows_out) throw std::runtime_error("dissipation_eta: null rows_out");
    if (m.cfg.model == SMC_MODEL_CONST) {
      *rows_out = 0;
    } else if (m.cfg.model == SMC_MODEL_ETA_T && m.have_last_eta) {
      copy_out(m, eta_out, m.dLastEta, mem, sizeof(double) * m.Nx * m.N);
      *rows_out = m.Nx;
    } else {
      copy_out(m, eta_out, m.dEzProf, mem, sizeof(double) * m.N);
      *rows_out = 1;
    }
  })
}

int smc_schur_matvec(smc_handle* h, const double* eta, const double* v, double* out, int mem) {
  SMC_GUARD(h, {
    Model& m = h->m;
    if (m.cfg.model != SMC_MODEL_ETA_T) throw std::runtime_error("schur_matvec needs the eta_T model");
    auto kin = mem == SMC_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    SMC_CUDA(cudaMemcpyAsync(m.dEta, eta, sizeof(double) * m.Nx * m.N, kin, m.stream));
    copy_in(m, m.dIn, v, mem, m.n);
    m.eta_operator();
    if (m.matvec_variant == 0) m.schur_matvec(m.dIn, m.dOut);
    else m.schur_matvec_fast(m.dIn, m.dOut, m.matvec_variant == 2);
    copy_out(m, out, m.dOut, mem, m.n * sizeof(double2));
  })
}

int smc_set_option(smc_handle* h, const char* key, double value) {
  SMC_GUARD(h, {
    std::string k(key ? key : "");
    if (k == "dense_mult_eta") h->m.use_dense_mult = value != 0.0;
    else if (k == "schur_matvec_variant") {
      int v = (int)value;
      if (v < 0 || v > 2) throw std::runtime_error("schur_matvec_variant must be 0, 1 or 2");
      if (v > 0 && !h->m.fast) throw std::runtime_error("fused variants need a SMC_MIXED handle");
      h->m.matvec_variant = v;
    } else if (k == "inner_fp32") {
      h->m.inner_fp32 = value != 0.0;
    } else if (k == "krylov_engine") {
      h->m.use_engine = value != 0.0;
    } else if (k == "bfbt_reuse_rel" || k == "bfbt_reuse_age") {
      if (h->m.bfbt_exec) throw std::runtime_error(k + ": set it before the first Stokes solve");
      if (k == "bfbt_reuse_rel") {
        if (!(value >= 0.0 && value < 1.0)) throw std::runtime_error("bfbt_reuse_rel must be in [0, 1)");
        h->m.bfbt_reuse_rel = value;
      } else {
        if (!(value >= 1.0 && value <= 1e6)) throw std::runtime_error("bfbt_reuse_age must be in [1, 1e6]");
        h->m.bfbt_reuse_age = (int)value;
      }
    } else if (k == "theta_precond_lag") {
      if (!(value >= 0.0 && value < 1.0)) throw std::runtime_error("theta_precond_lag must be in [0, 1)");
      h->m.theta_lag = value;
    } else if (k == "inner_rtol_floor" || k == "stokes_inner_rtol_floor" ||
               k == "theta_inner_rtol_floor") {
      if (!(value > 0.0 && value < 1.0)) throw std::runtime_error(k + " must be in (0, 1)");
      if (k[0] != 't') h->m.inner_floor[0] = value;
      if (k[0] != 's') h->m.inner_floor[1] = value;
    } else if (k == "engine_ctas") {
      if (!(value >= 0.0 && value <= 1e6)) throw std::runtime_error("engine_ctas must be >= 0");
      h->m.eng_ctas = (int)value;
    } else if (k == "engine_phase_profile") {
      h->m.eng_phase = value != 0.0;
    } else if (k == "warm_start") {
      h->m.warm_start = value != 0.0;
    } else if (k == "warm_extrapolate") {
      if (!(value >= 0.0 && value <= 3.0)) throw std::runtime_error("warm_extrapolate must be 0..3");
      h->m.warm_extrap = (int)value;
    } else if (k == "tc_transforms") {
      h->m.enable_tc(value != 0.0);
    } else if (k == "tc_lu") {
      h->m.enable_tc_lu(value != 0.0);
    } else if (k == "engine_batch") {
      h->m.enable_batch(value != 0.0);
    } else if (k == "engine_batch_ctas") {
      if (!(value >= 0.0 && value <= 1e6)) throw std::runtime_error("engine_batch_ctas must be >= 0");
      h->m.batch_ctas = (int)value;
    } else if (k == "engine_batch_hold_us") {
      if (!(value >= 0.0 && value <= 1e6)) throw std::runtime_error("engine_batch_hold_us must be >= 0");
      smc::batch_set_hold_us(h->m.device, value);
    } else if (k == "engine_batch_refill") {
      smc::batch_set_refill(h->m.device, value != 0.0 ? 1 : 0, -1.0, -1.0);
    } else if (k == "engine_batch_idle_us" || k == "engine_batch_life_us") {
      if (!(value >= 0.0 && value <= 1e7)) throw std::runtime_error(k + " must be >= 0");
      smc::batch_set_refill(h->m.device, 1, k == "engine_batch_idle_us" ? value : -1.0,
                            k == "engine_batch_life_us" ? value : -1.0);
    } else if (k == "engine_batch_gpu_ctas") {
      if (!(value >= 0.0 && value <= 1e6)) throw std::runtime_error("engine_batch_gpu_ctas must be >= 0");
      smc::batch_set_cap(h->m.device, (int)value);
    } else throw std::runtime_error("unknown option " + k);
  })
}

int smc_reset_history(smc_handle* h) {
  SMC_GUARD(h, { h->m.have_prev = false; })
}

int smc_get_history(smc_handle* h, double* prev_out, double* psi_prev_out, int mem,
                    double* dt_prev, int* have_prev) {
  SMC_GUARD(h, {
    Model& m = h->m;
    if (!prev_out || !psi_prev_out || !dt_prev || !have_prev)
      throw std::runtime_error("smc_get_history: null pointer");
    copy_out(m, prev_out, m.dPrev, mem, m.n * sizeof(double2));
    copy_out(m, psi_prev_out, m.dPsiPrev, mem, m.n * sizeof(double2));
    *dt_prev = m.dt_prev;
    *have_prev = m.have_prev ? 1 : 0;
  })
}

int smc_set_history(smc_handle* h, const double* prev, const double* psi_prev, int mem,
                    double dt_prev, int have_prev) {
  SMC_GUARD(h, {
    Model& m = h->m;
    if (have_prev) {
      if (!prev || !psi_prev) throw std::runtime_error("smc_set_history: null pointer");
      if (!(dt_prev > 0.0)) throw std::runtime_error("smc_set_history: dt_prev must be > 0");
      copy_in(m, m.dPrev, prev, mem, m.n);
      copy_in(m, m.dPsiPrev, psi_prev, mem, m.n);
      SMC_CUDA(cudaStreamSynchronize(m.stream));
    }
    m.dt_prev = have_prev ? dt_prev : 0.0;
    m.have_prev = have_prev != 0 && m.cfg.model != SMC_MODEL_CONST;
  })
}

int smc_counters_get(smc_handle* h, smc_counters* out) {
  SMC_GUARD(h, {
    Model& m = h->m;
    *out = m.ctr;
    out->n_kernel_launches = m.nlaunch;
    // the viscosity pipeline's counters accumulate on the device
    smc::EtaCtrDev* d = reinterpret_cast<smc::EtaCtrDev*>(m.hbuf);
    SMC_CUDA(cudaMemcpyAsync(d, m.dEtaCtr, sizeof(smc::EtaCtrDev), cudaMemcpyDeviceToHost, m.stream));
    SMC_CUDA(cudaStreamSynchronize(m.stream));
    out->n_T_out_of_range += d->n_T_out_of_range;
    out->n_clip_T += d->n_clip_T;
    out->n_clip_eta += d->n_clip_eta;
    out->n_smooth_eta += d->n_smooth_eta;
    out->n_clip_eta_proj += d->n_clip_eta_proj;
    out->n_smooth_eta_proj += d->n_smooth_eta_proj;
    out->max_T_excursion = std::max(out->max_T_excursion, d->max_T_excursion);
  })
}

int smc_shape(smc_handle* h, int* Nk, int* Nx, int* Nz, int* Np) {
  SMC_GUARD(h, {
    *Nk = h->m.Nk; *Nx = h->m.Nx; *Nz = h->m.N; *Np = h->m.Np;
  })
}

void* smc_stream(smc_handle* h) { return h ? (void*)h->m.stream : nullptr; }

const char* smc_last_error(void) { return smc::g_last_error.c_str(); }

}  // extern "C"

// ------------------------------------------------------------------ many runs
namespace smc {

// out[0] = max |g|, out[1] = number of non-finite entries (one CTA)
__global__ void smc_maxabs_finite_kernel(const double* __restrict__ g, long long n,
                                         double* __restrict__ out) {
  __shared__ double sm[32];
  __shared__ int sb[32];
  double m = 0.0;
  int bad = 0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const double v = g[i];
    if (!isfinite(v)) ++bad;
    else m = fmax(m, fabs(v));
  }
  for (int o = 16; o > 0; o >>= 1) {
    m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    bad += __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) { sm[threadIdx.x >> 5] = m; sb[threadIdx.x >> 5] = bad; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    int b = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { a = fmax(a, sm[w]); b += sb[w]; }
    out[0] = a;
    out[1] = (double)b;
  }
}

// max |theta| on the (Nx, Nz) grid of the resident state; -1 if any value
// of the state's grid is not finite
double resident_amplitude(Model& m) {
  const double2* cur = m.resident_cur0 ? m.dS0 : m.dS1;
  m.synth(cur, m.dV, KFactor(), m.gr[0], m.Nx, m.sp[0]);
  smc_maxabs_finite_kernel<<<1, 512, 0, m.stream>>>(m.gr[0], (long long)m.Nx * m.N, m.dScal);
  SMC_LAUNCH_CHECK(m.ctx);
  m.sync_read(m.dScal, 2);
  return m.hbuf[1] > 0.0 ? -1.0 : m.hbuf[0];
}

}  // namespace smc

int smc_create_many(const smc_config* cfgs, int nruns, smc_handle** out) {
  if (!cfgs || !out || nruns < 0) {
    smc::set_last_error("smc_create_many: null argument or negative count");
    return -1;
  }
  for (int i = 0; i < nruns; ++i) out[i] = nullptr;
  for (int i = 0; i < nruns; ++i) {
    const int rc = smc_create(&cfgs[i], &out[i]);
    if (rc != 0) {
      const std::string msg = "run " + std::to_string(i) + ": " + smc_last_error();
      for (int j = 0; j < i; ++j) { smc_destroy(out[j]); out[j] = nullptr; }
      smc::set_last_error(msg.c_str());
      return rc;
    }
  }
  return 0;
}

int smc_march_many(smc_handle* const* hs, int nruns, long long nsteps, double safety,
                   double dtmax, double amp_limit, int check_every, int concurrency,
                   int batched, smc_run_result* res) {
  using namespace smc;
  try {
    if (!hs || !res || nruns < 0) throw std::runtime_error("smc_march_many: null argument");
    for (int i = 0; i < nruns; ++i)
      if (!hs[i]) throw std::runtime_error("smc_march_many: null handle " + std::to_string(i));
    if (check_every < 1) check_every = 1;
    if (concurrency < 1) concurrency = 1;
    concurrency = std::min(concurrency, std::max(nruns, 1));
    for (int i = 0; i < nruns; ++i) {
      Model& m = hs[i]->m;
      if (batched && m.fast) {
        SMC_CUDA(cudaSetDevice(m.device));
        m.enable_batch(true);
      }
    }
    std::atomic<int> next{0};
    std::mutex err_mu;
    std::string first_err;
    auto worker = [&]() {
      while (true) {
        const int i = next.fetch_add(1);
        if (i >= nruns) break;
        smc_run_result& r = res[i];
        std::memset(&r, 0, sizeof(r));
        r.status = SMC_RUN_OK;
        Model& m = hs[i]->m;
        try {
          SMC_CUDA(cudaSetDevice(m.device));
          BatchScope bs(m.device, m.batch_mode);
          const auto t0 = std::chrono::steady_clock::now();
          r.amp0 = resident_amplitude(m);
          r.amp = r.amp0;
          if (r.amp0 < 0.0) r.status = SMC_RUN_NONFINITE;
          smc_march_info info{};
          while (r.status != SMC_RUN_NONFINITE && r.steps < nsteps) {
            const long long k = std::min<long long>(check_every, nsteps - r.steps);
            advance_resident(m, INFINITY, k, safety, dtmax, &info);
            m.settle();
            m.check_tc();
            r.steps += info.steps;
            r.t = info.t;
            r.dt = info.dt;
            const double a = resident_amplitude(m);
            if (a < 0.0 || !std::isfinite(info.t)) { r.status = SMC_RUN_NONFINITE; break; }
            r.amp = a;
            if (r.status == SMC_RUN_OK && amp_limit > 0.0 && a > amp_limit * r.amp0)
              r.status = SMC_RUN_AMPLITUDE;
            if (info.steps < k) break;
          }
          r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        } catch (const std::exception& e) {
          r.status = SMC_RUN_ERROR;
          std::lock_guard<std::mutex> lk(err_mu);
          if (first_err.empty()) first_err = "run " + std::to_string(i) + ": " + e.what();
        }
      }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < concurrency; ++t) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    if (!first_err.empty()) throw std::runtime_error(first_err);
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}

int smc_batch_stats(int device, long long* launches, long long* solves, long long* ctas) {
  try {
    smc::batch_stats(device, launches, solves, ctas);
    return 0;
  } catch (const std::exception& e) {
    return fail(e);
  }
}
