// Persistent on-device FGMRES of the fast form (smc_engine.cu).
#pragma once
#include "smc_internal.cuh"

namespace smc {

// Operator + preconditioner of one engine solve.  Arrays typed T (the
// working precision) are passed as void*; kind 0 = fused Schur matvec,
// kind 1 = fused temperature matvec.  The dense operator matrices are
// stored TRANSPOSED (column index outermost) so that a warp reads 32
// consecutive output rows of one column in one coalesced access.
struct EngineOps {
  int kind = 0;
  int Nk = 0, N = 0, Mz = 0, L = 0, Np = 0;
  // Schur operator (T): z-contraction [q][s] (Zf shared by all k; Z1..Z3 per
  // k, [k][q][s]), epilogue [q][p], x-convolution weights E [l][s], twiddles
  const void *ZfT = nullptr, *Z1T = nullptr, *Z2T = nullptr, *Z3T = nullptr;
  const void *D2ZiT = nullptr, *ZiT = nullptr, *DZiT = nullptr;
  const void *E = nullptr, *twS = nullptr;
  // T = float: Zf, Z1 and D2Zi also as (hi, lo) float pairs, same layouts.  The
  // eta v and 2 k^2 eta G v fields are differentiated twice by the epilogue,
  // which amplifies rounding in their point values: those two contractions
  // and the D2Zi product are summed in double-float arithmetic (FP32 ones
  // leave the FP32 operator ~1e-1 from the FP64 one in the residual norm,
  // these ~3e-3, so each refinement pass gains that much more)
  const void *ZfT2 = nullptr, *Z1T2 = nullptr, *D2ZiT2 = nullptr;
  // temperature operator (T): z-synthesis [q][j], epilogue [m][n], twiddles,
  // frozen velocities on the padded grid
  const void *tVT = nullptr, *tVDT = nullptr, *tD2T = nullptr, *tViT = nullptr, *twT = nullptr;
  const void *ux = nullptr, *uz = nullptr;
  double a0 = 0.0;
  const void* kxT = nullptr;          // kx in T
  const double* kx = nullptr;         // kx in FP64
  const double* V64 = nullptr;        // FP64 basis (tau rows)
  // preconditioner: z_k = palpha * G_k v_k, G stored transposed [k][m][n]:
  // FP64 values for T = double; (hi, lo) float pairs for T = float, applied
  // in double-float arithmetic (the products G_k v cancel too strongly for
  // plain FP32 on the later refinement corrections)
  const void* GpT = nullptr;
  double palpha = 1.0;
  // scratch (T complex): Fv/Hv (4 Nk Mz), X (2 Nk N), A (Nk N)
  void *Fv = nullptr, *Hv = nullptr, *X = nullptr, *A = nullptr;
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
  double* npart = nullptr;   // 2 * max_grid
  int* flag = nullptr;
  int* result = nullptr;     // {info, iterations}
  int max_grid = 0;
  int grid_cap = 0;          // > 0: at most this many CTAs (handles sharing the GPU)
  // optional: SM cycles CTA 0 spent between consecutive grid barriers, summed
  // per phase (ENGINE_PHASES slots, names in engine_phase_names); null = off
  long long* phase_cycles = nullptr;
};

// phases of one Arnoldi step (and of a restart cycle) between grid barriers;
// the *_WAIT slots hold CTA 0's wait at the grid barrier that ends the phase,
// the others its own work
enum EnginePhase {
  EP_START = 0,  // V0 = r / beta, its preconditioned vector and z-contraction
  EP_XCONV,      // x-direction convolution (per z-point / grid column)
  EP_XCONV_WAIT,
  EP_POST,       // operator epilogue + first-pass orthogonalisation dots
  EP_POST_WAIT,
  EP_UPD_RED,    // reduction of the first-pass dots
  EP_UPDATE,     // first-pass update + second-pass dots + ||w'||^2
  EP_UPDATE_WAIT,
  EP_EXACT,      // exact norm after heavy cancellation (rare)
  EP_NEXT_RED,   // reduction of the second-pass dots and of ||w'||^2
  EP_GIVENS,     // Givens update of the new Hessenberg column
  EP_COMBINE,    // next basis row v = (w' - V h2) / h
  EP_PRECOND,    // its preconditioned row
  EP_CONTRACT,   // z-contraction slice
  EP_NEXT_WAIT,
  EP_LSQ,        // triangular solve + x update at the end of a cycle
  EP_RESID,      // true residual at a restart
  // outer pass of the refinement engine: x += e, then r = b - A64 x in the
  // FP64 operator phases, then ||r||
  EP_REF_XUPD,
  EP_REF_PREP,   // FP64 z-contraction of x
  EP_REF_XCONV,  // FP64 x-direction convolution
  EP_REF_POST,   // FP64 epilogue r = b - A x and ||r||^2 partials
  EP_REFINE,     // ||r|| reduction
  // whole launch as seen by CTA 0: SM cycles and %globaltimer nanoseconds
  // (their ratio is the SM clock the engine ran at)
  EP_TOTAL_CYCLES,
  EP_TOTAL_NS,
  ENGINE_PHASES
};
extern const char* const engine_phase_names[2][ENGINE_PHASES];

void fgmres_engine(const Ctx& c, const EngineOps& op, const EngineIO& io, bool fp32);

// The outer loop of FP32-inner / FP64-outer iterative refinement, on the device
struct RefineIO {
  const double2* b = nullptr;   // right-hand side (FP64)
  double2* x = nullptr;         // solution (FP64)
  double2* r = nullptr;         // outer residual scratch (FP64, n)
  double2* e = nullptr;         // inner correction scratch (FP64, n)
  double rtol = 1e-8;           // outer relative tolerance
  double floor = 1e-4;          // smallest inner relative tolerance
  int maxiter = 800;            // inner Arnoldi steps in all
  double* res = nullptr;        // -> final relative residual (device)
  int warm = 0;                 // 1: x holds the initial guess (else x starts at 0)
};
// io: the engine workspace; io.result -> {info, inner steps, outer passes}
void fgmres_refine_engine(const Ctx& c, const EngineOps& op32, const EngineOps& op64,
                          const EngineIO& io, const RefineIO& rf);

// ------------------------------------------------------ batched refinement
// Result block of one batched solve, in host-mapped pinned memory: the
// kernel writes the fields, then (after a system-scope fence) `done` = the
// job's sequence number, which the owning host thread polls.
struct EngineJobResult {
  volatile int done;
  int info, iters, outer, failed;
  double rel;
};

// One solve of a batched launch: the operators and workspace of its handle
// (exactly what fgmres_refine_engine takes), the CTA range [cta0, cta0 + G)
// of its slot when it is a slot's first solve, and the device address of its
// result block.
struct RefineJob {
  EngineOps op32, op64;
  EngineIO io;
  RefineIO rf;
  EngineJobResult* out = nullptr;
  int seq = 0;
  int cta0 = 0, G = 0;
};

constexpr int ENGINE_BATCH_MAX = 16;
constexpr int BATCH_FEED_CAP = 256;

// Solves handed to a running batch (host-mapped pinned memory): the host
// writes ring[i] and then, after a release fence, published = i + 1; a group
// that has finished its solve claims the next ticket (a device counter) and
// runs that solve on its own CTAs.
struct BatchFeed {
  volatile int published;
  int pad[63];
  RefineJob ring[BATCH_FEED_CAP];
};

struct RefineBatch {
  RefineJob job[ENGINE_BATCH_MAX];   // the first solve of each group (slot)
  int njobs = 0;
  int* err = nullptr;             // raised when any group barrier timed out
  long long timeout_ns = 2000000000LL;
  unsigned int* slot_bar = nullptr;  // 4 zeroed words per slot: arrivals, generation, time-out
  // refill: null feed = each group runs its first solve only
  BatchFeed* feed = nullptr;         // device address of the host-mapped feed
  int* claimed = nullptr;            // tickets taken (device, zero at launch)
  int* slot_ticket = nullptr;        // per slot: the ticket its leader claimed (-1: none)
  long long idle_ns = 200000;        // a group leaves after this long without a queued solve
  long long life_ns = 20000000;      // no solve is claimed after this long (other cooperative
                                     // kernels wait for the launch to end)
};

// dynamic shared memory of a refinement solve (the larger of its two operators)
size_t refine_engine_smem(const EngineOps& op32, const EngineOps& op64);
// co-resident CTAs of the batched kernel at `smem` bytes of dynamic smem
int refine_batch_capacity(size_t smem, int num_sms);
// one cooperative launch of the jobs of B (cta0 contiguous from 0) on stream s
void refine_batch_launch(cudaStream_t s, const RefineBatch& B, size_t smem);

// out[b][c][r] = (To) in[b][r][c] for batch matrices of rows x cols
void transpose_as(const Ctx& c, const double* in, float* out, long long rows, long long cols, int batch);
void transpose_as(const Ctx& c, const double* in, double* out, long long rows, long long cols, int batch);
// out[b][c][r] = (hi, lo) with hi = (float) in[b][r][c], lo = (float)(in - hi)
void transpose_split(const Ctx& c, const double* in, float2* out, long long rows, long long cols,
                     int batch);

}  // namespace smc
