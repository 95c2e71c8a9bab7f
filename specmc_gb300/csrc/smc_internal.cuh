// Internal declarations shared by the translation units of libspecmc_gb300.
//
// Layout conventions (device memory):
//   spectral fields   (Nk, Nz) complex  row-major, double2 / float2 (re, im)
//   grid fields       (Ng, Nz) real     row-major (x node i, CGL node j)
//   small operators   (N, N) real       row-major unless a name says "cm"
//                                       (column-major, used by LU factors)
//   dense Schur LU    (n, n) complex    column-major, n = Nk * Nz
#pragma once
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>
#include <cstdint>
#include <stdexcept>
#include <string>

namespace smc {

// ------------------------------------------------------------------ errors
struct CudaError : std::runtime_error {
  explicit CudaError(const std::string& m) : std::runtime_error(m) {}
};

#define SMC_CUDA(call)                                                        \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess)                                                    \
      throw ::smc::CudaError(std::string(#call) + ": " +                      \
                             cudaGetErrorString(e_) + " (" + __FILE__ + ":" + \
                             std::to_string(__LINE__) + ")");                 \
  } while (0)

// Optional per-tag event timer: when enabled, the launch helpers bracket
// the kernels of a tag with CUDA events on the handle's stream; elapsed
// times are resolved (and the events recycled) by Profiler::resolve.
struct Profiler {
  static constexpr int MAXTAG = 64;
  bool enabled = false;
  bool engine_only = false;       // time only the Krylov engine regions ("engine_*")
  bool wants(const char* name) const {
    return enabled && (!engine_only || std::strncmp(name, "engine_", 7) == 0);
  }
  const char* names[MAXTAG] = {nullptr};
  double ms[MAXTAG] = {0};
  long long launches[MAXTAG] = {0};
  double work[MAXTAG] = {0};      // algorithmic flops or bytes, as tagged
  int work_is_bytes[MAXTAG] = {0};
  struct Pending { int tag; cudaEvent_t a, b; };
  Pending* pend = nullptr;
  int npend = 0, cap = 0;
  cudaEvent_t* pool = nullptr;
  int npool = 0;
  int tag_of(const char* name);
  void begin(cudaStream_t s, int tag, cudaEvent_t* a);
  void end(cudaStream_t s, int tag, cudaEvent_t a, double work_amount, int is_bytes);
  void resolve();
  void reset();
  // a region timed on the device by other means (ms, launch count)
  void add(const char* name, double ms_, long long n_);
  // work of a region known only after its launch (a deferred engine result)
  void add_work(const char* name, double w) {
    if (wants(name)) work[tag_of(name)] += w;
  }
  ~Profiler();
};

struct TcCache;

// Launch context: the stream every kernel of a handle goes to, the launch
// counter the handle reports, the optional profiler, and the tensor-core
// operators of the z-contractions (null: FP64 SIMT contractions only).
struct Ctx {
  cudaStream_t s = nullptr;
  long long* nlaunch = nullptr;
  int num_sms = 152;
  Profiler* prof = nullptr;
  TcCache* tc = nullptr;
  void count(int n = 1) const { if (nlaunch) *nlaunch += n; }
};

// RAII bracket of one tagged launch region
struct ProfScope {
  const Ctx& c;
  int tag = -1;
  cudaEvent_t a = nullptr;
  double work;
  int is_bytes;
  ProfScope(const Ctx& c_, const char* name, double work_ = 0.0, int is_bytes_ = 0)
      : c(c_), work(work_), is_bytes(is_bytes_) {
    if (c.prof && c.prof->wants(name)) {
      tag = c.prof->tag_of(name);
      c.prof->begin(c.s, tag, &a);
    }
  }
  ~ProfScope() {
    if (tag >= 0) c.prof->end(c.s, tag, a, work, is_bytes);
  }
};

#define SMC_LAUNCH_CHECK(ctx)                                                 \
  do {                                                                        \
    (ctx).count();                                                            \
    cudaError_t e_ = cudaGetLastError();                                      \
    if (e_ != cudaSuccess)                                                    \
      throw ::smc::CudaError(std::string("kernel launch: ") +                 \
                             cudaGetErrorString(e_) + " (" + __FILE__ + ":" + \
                             std::to_string(__LINE__) + ")");                 \
  } while (0)

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Cooperative grids (grid-wide or group barriers) never overlap on a GPU: a
// cooperative kernel needs all of its CTAs resident at once, and two of them
// each holding SMs while waiting for the rest of their own CTAs would never
// finish.  Every cooperative launch of the process is made under one lock and
// ordered on the GPU after the previous one of the same device (any stream)
// by an event: the launch's stream waits for the event, the launch records
// it.  So no host thread waits for a cooperative kernel to finish just to
// release the lock, and ordinary kernels of other streams keep running beside
// it.
std::mutex& coop_mutex();
// inside the lock: order stream s after the device's last cooperative launch /
// record the launch just made on s as the device's last one
void coop_order_before(cudaStream_t s);
void coop_order_after(cudaStream_t s);

// Let kernel `f` use up to the device's opt-in maximum of dynamic shared
// memory.  The attribute is global to the process, so every caller sets the
// same value (a smaller per-launch value set by one handle could otherwise
// undercut another handle's launch in between).
void allow_max_smem(const void* f);
struct CoopGuard {
  cudaStream_t s;
  std::unique_lock<std::mutex> lk;
  explicit CoopGuard(cudaStream_t s_) : s(s_), lk(coop_mutex()) { coop_order_before(s); }
  ~CoopGuard() { coop_order_after(s); }
};

// ------------------------------------------------------- complex helpers
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) {
  return make_double2(a.x + b.x, a.y + b.y);
}
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) {
  return make_double2(a.x - b.x, a.y - b.y);
}
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) {
  return make_double2(a.x * s, a.y * s);
}
__host__ __device__ __forceinline__ double2 cconj(double2 a) {
  return make_double2(a.x, -a.y);
}
// numpy-style complex division (Smith's algorithm is what CPython uses for
// complex128 true division; the exact formula only matters at roundoff level)
__host__ __device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  double ar = fabs(b.x), ai = fabs(b.y);
  if (ar >= ai) {
    double r = b.y / b.x, d = b.x + b.y * r;
    return make_double2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  }
  double r = b.x / b.y, d = b.y + b.x * r;
  return make_double2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
__host__ __device__ __forceinline__ double cabs1(double2 a) {  // |re| + |im|
  return fabs(a.x) + fabs(a.y);
}

// per-mode complex factor (cre + i cim) * kx[k]^kpow
struct KFactor {
  double cre = 1.0, cim = 0.0;
  int kpow = 0;
};

__device__ __forceinline__ double2 kfactor_eval(const KFactor& f, double kx) {
  double p = 1.0;
  for (int e = 0; e < f.kpow; ++e) p *= kx;
  return make_double2(f.cre * p, f.cim * p);
}

// ============================================================ spectral ops
// Y_b[k][n] (=|+=) f_b(k) * sum_m Z_b[n][m] X_b[k][m]   (Z real N x N;
// per-k operator when zstride > 0).  Up to 4 jobs per launch.
// Sums split over consecutive lanes (the FP64 contractions and x-direction
// DFTs, see smc_zmat_kernel; ZSPLIT lanes per column in the Green-column
// solves): the lane partials combined pairwise, (p0 + p1) + (p2 + p3) for 4
// lanes and ((p0 + p1) + (p2 + p3)) + ((p4 + p5) + (p6 + p7)) for CSPLIT = 8,
// the same value in every lane of the group
constexpr int ZSPLIT = 4;
constexpr int CSPLIT = 8;
__device__ __forceinline__ double split4_sum(double v) {
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  return v;
}
__device__ __forceinline__ double split8_sum(double v) {
  v = split4_sum(v);
  v += __shfl_xor_sync(0xffffffffu, v, 4);
  return v;
}

struct ZJob {
  const double* Z = nullptr;
  long long zstride = 0;
  const double2* X = nullptr;
  double2* Y = nullptr;
  KFactor f;
  int accumulate = 0;
  int x_real = 0;        // use Re(X) only
  int zero_tau = 0;      // write 0 to columns N-2, N-1 of Y
};
void zmat_apply(const Ctx& c, const ZJob* jobs, int njobs, int Nk, int N,
                const double* kx);

// g_b[i][j] = sum_k w_k Re(X_b[k][j] e^{2 pi i k i / Ng})  (irfft * Ng)
struct SynthJob {
  const double2* X = nullptr;
  double* g = nullptr;
};
void synth_x(const Ctx& c, const SynthJob* jobs, int njobs, int Nk, int N,
             int Ng, const double2* tw);

// A_b[k][j] = scale * sum_i g_b[i][j] e^{-2 pi i k i / Ng},  k < Nk
struct AnaJob {
  const double* g = nullptr;
  double2* A = nullptr;
};
void analysis_x(const Ctx& c, const AnaJob* jobs, int njobs, int Nk, int N,
                int Ng, const double2* tw, double scale);

// elementwise kernels on grids (Ng * N points)
void grid_explicit_nonlinear(const Ctx& c, const double* ux, const double* uz,
                             const double* thx, const double* thz, double H,
                             double* out, long long npts);
void grid_advect_product(const Ctx& c, const double* ux, const double* uz,
                         const double* vx, const double* vz, double* out,
                         long long npts);
void grid_phi(const Ctx& c, const double* gxx, const double* gzz,
              const double* gxz, const double* gtr, const double* eta_pad,
              double coef, double* out_accum, long long npts, int accumulate);

// max|a|, max|b| (nullable b) -> dst[0]
void reduce_maxabs2(const Ctx& c, const double* a, const double* b, long long n,
                    double* dst, double* scratch);

// ============================================================ vector ops
// generic spectral combinations (n complex entries)
void vec_axpby(const Ctx& c, double2* y, double2 a, const double2* x, double2 b,
               long long n);                           // y = a x + b y
void vec_copy(const Ctx& c, double2* y, const double2* x, long long n);
void vec_zero(const Ctx& c, void* p, long long bytes);
// out[k][n] = alpha*in[k][n]  with tau columns forced to 0 and row kx==0
// forced to 0 when zero_k0
void vec_scaled_modes(const Ctx& c, const double2* in, double2* out, int Nk,
                      int N, KFactor f, const double* kx, int zero_tau,
                      int zero_k0);
// dot / norm reductions (partials in scratch, result at dst)
void vec_norm2(const Ctx& c, const double2* x, long long n, double* dst,
               double* scratch);
// memo signature test of the coupled model: dst = {all_equal, max|X-cX|, max|cX|}
void memo_compare(const Ctx& c, const double2* that, const double2* cthat,
                  const double2* X, const double2* cX, long long n, double* dst,
                  double* scratch);

// ============================================================ dense ops
// in-place LU with partial pivoting of `count` real N x N matrices
// (column-major, stride N*N); piv 0-based LAPACK ipiv; info[b] = first zero pivot+1
void lu_small_batched(const Ctx& c, double* A, int* piv, int* info, int N,
                      int count);
// the same factorisation of A (may equal LU) into LU / piv, then the
// explicit inverse operators G_k = A_k^{-1} P (P: identity with rows N-2, N-1
// zeroed) from the factors over several CTAs per matrix: G row-major, GT64
// its transpose, GT32 the transpose as (hi, lo) floats, each when not null.
// False, with nothing launched, for N > 96 (the callers then run
// green_from_lu and the transposes).
bool lu_green_batched(const Ctx& c, const double* A, double* LU, int* piv, double* G,
                      double* GT64, float2* GT32, int N, int count);
// x_b = A_b^{-1} (alpha * P b_b): P zeroes rows N-2, N-1 when zero_tau
void lu_small_solve(const Ctx& c, const double* LU, const int* piv, long long lu_stride,
                    const double2* b, double2* x, int N, int count, double alpha,
                    int zero_tau, const int* skip_mask);
// dense complex LU (column-major n x n) with partial pivoting (|re|+|im| pivot
// choice, as LAPACK zgetrf); piv 0-based.  With tcwork (tclu_work_bytes(n)
// bytes) the trailing updates run on the tensor cores (smc_tclu.cu, FP64
// accuracy; *tcerr raised if one of its CTAs timed out)
void zlu_dense(const Ctx& c, double2* A, int* piv, int n, double2* work, void* tcwork = nullptr,
               int* tcerr = nullptr);
size_t tclu_work_bytes(int n);
void tclu_update(const Ctx& c, double2* A, int n, int p0, int nbp, void* work, int* err);
// inverses of the 64 x 64 diagonal blocks of L and U (column-major blocks)
void zlu_diag_inverses(const Ctx& c, const double2* LU, int n, double2* invL, double2* invU);
// x = A^{-1} b with a zlu_dense factor; perm = composed row permutation;
// work: n complex
void zlu_dense_solve(const Ctx& c, const double2* LU, const double2* invL, const double2* invU,
                     const int* perm, const double2* b, double2* x, int n, double2* work);

// ============================================================ Schur ops
// complex Chebyshev product matrices M_d for d in (-Nk, Nk): Md[(d+Nk-1)] (N x N row-major)
void build_mult_mats(const Ctx& c, const double2* eta_c, double2* Md, int Nk, int N);
// out = mult_eta(f) (one-sided convolution + partner half with sign sgn)
void mult_eta(const Ctx& c, const double2* Md, const double2* f, double2* out,
              int Nk, int N, double sgn, double2* partial);
// dense Schur assembly (column-major) from Md, D, D2, G, V
void assemble_schur(const Ctx& c, const double2* Md, const double* D,
                    const double* D2, const double* G, const double* V,
                    const double* kx, double2* A, int Nk, int N, double2* work);

}  // namespace smc
