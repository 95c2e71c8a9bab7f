// Dense linear algebra of the FP64 time step.
//
//  * Batched small LU (one CTA per matrix, the matrix held in shared memory)
//    for the per-wavenumber operators of SpecMC: the Chebyshev-tau Helmholtz
//    operators (rbc_galerkin.py:119-185), the reduced eta(z) Stokes operators
//    (stokes/vv_stokes.py:298-321) and the BFBT blocks (stokes/bfbt.py:157-191).
//  * Blocked right-looking complex LU with partial pivoting and the matching
//    triangular solve for the lagged dense Schur matrix (lagged_stokes.py:
//    274-300, scipy lu_factor / lu_solve).  The pivot of each column is the
//    first row of largest |re| + |im|, the choice LAPACK's zgetrf makes.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so every FP64 kernel
// here spreads its arithmetic over all SMs: the panel factorisation and the
// triangular solves are single cooperative launches (one CTA per SM) that
// synchronise the grid between dependent steps, and the trailing update is a
// tiled GEMM over the whole machine.
#include <cooperative_groups.h>

#include "smc_internal.cuh"
#include "smc_schur.cuh"

namespace cg = cooperative_groups;

namespace smc {

// ======================================================== small batched LU
__global__ void smc_lu_small_kernel(double* __restrict__ A, int* __restrict__ piv,
                                    int* __restrict__ info, int N) {
  extern __shared__ double a[];                   // N*N column-major
  __shared__ double rv[32];
  __shared__ int ri[32];
  __shared__ int s_p;
  const int tid = threadIdx.x, nt = blockDim.x;
  double* Ag = A + (long long)blockIdx.x * N * N;
  for (int i = tid; i < N * N; i += nt) a[i] = Ag[i];
  __syncthreads();
  int inf = 0;
  for (int c = 0; c < N; ++c) {
    // pivot: first row of largest |a[r,c]|, r >= c (idamax)
    double best = -1.0;
    int bi = N;
    for (int r = c + tid; r < N; r += nt) {
      double v = fabs(a[r + c * N]);
      if (v > best) { best = v; bi = r; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      double ov = __shfl_xor_sync(0xffffffffu, best, o);
      int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if ((tid & 31) == 0) { rv[tid >> 5] = best; ri[tid >> 5] = bi; }
    __syncthreads();
    if (tid == 0) {
      double b = rv[0];
      int p = ri[0];
      for (int w = 1; w < (nt >> 5); ++w)
        if (rv[w] > b || (rv[w] == b && ri[w] < p)) { b = rv[w]; p = ri[w]; }
      if (p >= N) p = c;
      s_p = p;
      piv[(long long)blockIdx.x * N + c] = p;
    }
    __syncthreads();
    const int p = s_p;
    if (p != c)
      for (int col = tid; col < N; col += nt) {
        double t = a[c + col * N];
        a[c + col * N] = a[p + col * N];
        a[p + col * N] = t;
      }
    __syncthreads();
    const double pv = a[c + c * N];
    if (pv != 0.0) {
      const double rinv = 1.0 / pv;
      for (int r = c + 1 + tid; r < N; r += nt) a[r + c * N] *= rinv;
    } else if (!inf) {
      inf = c + 1;
    }
    __syncthreads();
    // rank-1 update of the trailing block: lanes over rows, the CTA's warps
    // over columns (each element gets the same single update per step)
    {
      const int nw = nt >> 5, lane = tid & 31;
      for (int col = c + 1 + (tid >> 5); col < N; col += nw) {
        const double u = a[c + col * N];
        for (int r = c + 1 + lane; r < N; r += 32) a[r + col * N] -= a[r + c * N] * u;
      }
    }
    __syncthreads();
  }
  for (int i = tid; i < N * N; i += nt) Ag[i] = a[i];
  if (tid == 0 && info) info[blockIdx.x] = inf;
}

// bit-pattern tests: no FP64 instruction (GB300 issues those through a pipe
// of about two lanes per clock per SM, compares included)
__device__ __forceinline__ bool lus_zero(double v) { return (__double_as_longlong(v) << 1) == 0; }

// The explicit inverse operators G_k = A_k^{-1} P (P: the identity with the
// two tau columns zeroed, vv_stokes.py:281-296) from the factors: CTA (k, b)
// stages the factor of wavenumber k and the reciprocals of its diagonal in
// shared memory and solves 2 W columns of G_k (W warps), each warp two
// columns at a time with the columns in registers (lane l holds rows l,
// l + 32, ...) and x_c broadcast by shuffle: the row interchanges (exact on a
// unit vector: only the one moves), unit-lower forward substitution, upper
// back substitution multiplying by the reciprocal of the diagonal.  A step
// whose broadcast x_c is zero in both columns is skipped (it would change
// entries by signed zeros at most): the forward substitution of a column
// starts at the row its one moved to.  G is written row-major, its transpose
// (GT64) and the transpose as (hi, lo) float pairs (GT32), each when not null.
constexpr int GL_ROWS = 3;                         // rows a lane holds
constexpr int GL_MAXN = 32 * GL_ROWS;              // 96

template <int ROWS>
__device__ __forceinline__ double gl_pick(const double (&x)[ROWS], int j) {
  double v = x[0];
#pragma unroll
  for (int t = 1; t < ROWS; ++t)
    if (j == t) v = x[t];
  return v;
}

__global__ void __launch_bounds__(1024)
smc_green_lu_kernel(const double* __restrict__ LU, const int* __restrict__ piv, double* __restrict__ G,
                    double* __restrict__ GT64, float2* __restrict__ GT32, int N) {
  extern __shared__ double a[];                   // N*N factor of wavenumber k, then N reciprocals
  constexpr int ROWS = GL_ROWS;
  __shared__ int s_piv[GL_MAXN];
  double* rd = a + (long long)N * N;
  const int k = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long NN = (long long)N * N, kb = (long long)k * NN;
  for (int i = threadIdx.x; i < N * N; i += blockDim.x) a[i] = LU[kb + i];
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    s_piv[i] = piv[(long long)k * N + i];
    rd[i] = 1.0 / LU[kb + (long long)i * N + i];
  }
  __syncthreads();
  const int q0 = blockIdx.y * 2 * (blockDim.x >> 5) + 2 * warp, q1 = q0 + 1;
  if (q0 >= N) return;
  int pos0 = q0, pos1 = q1;
  for (int i = 0; i < N; ++i) {
    const int pi = s_piv[i];
    pos0 = pos0 == i ? pi : (pos0 == pi ? i : pos0);
    pos1 = pos1 == i ? pi : (pos1 == pi ? i : pos1);
  }
  double x0[ROWS], x1[ROWS];
#pragma unroll
  for (int j = 0; j < ROWS; ++j) {
    const int r = lane + 32 * j;
    x0[j] = r == pos0 ? 1.0 : 0.0;
    x1[j] = r == pos1 ? 1.0 : 0.0;
  }
  // (row chunks that need no update are skipped by warp-uniform branches: a
  // warp-wide FP64 instruction costs its 32 lanes whatever the predicate)
  for (int c = min(pos0, pos1); c < N; ++c) {     // unit lower
    const int cj = c >> 5, cl = c & 31;
    const double xc0 = __shfl_sync(0xffffffffu, gl_pick(x0, cj), cl);
    const double xc1 = __shfl_sync(0xffffffffu, gl_pick(x1, cj), cl);
    if (lus_zero(xc0) && lus_zero(xc1)) continue;
#pragma unroll
    for (int j = 0; j < ROWS; ++j) {
      if (32 * j + 31 <= c) continue;
      const int r = lane + 32 * j;
      const double l = (r > c && r < N) ? a[r + c * N] : 0.0;
      const bool need = !lus_zero(l);
      if (__any_sync(0xffffffffu, need) && need) {
        x0[j] -= l * xc0;
        x1[j] -= l * xc1;
      }
    }
  }
  for (int c = N - 1; c >= 0; --c) {              // upper
    const int cj = c >> 5, cl = c & 31;
    double xc0 = __shfl_sync(0xffffffffu, gl_pick(x0, cj), cl);
    double xc1 = __shfl_sync(0xffffffffu, gl_pick(x1, cj), cl);
    if (lus_zero(xc0) && lus_zero(xc1)) continue;
    const double r_c = rd[c];
    xc0 *= r_c;
    xc1 *= r_c;
#pragma unroll
    for (int j = 0; j < ROWS; ++j) {
      if (32 * j > c) continue;
      const int r = lane + 32 * j;
      if (r == c) {
        x0[j] = xc0;
        x1[j] = xc1;
      }
      const double u = r < c ? a[r + c * N] : 0.0;
      const bool need = !lus_zero(u);
      if (__any_sync(0xffffffffu, need) && need) {
        x0[j] -= u * xc0;
        x1[j] -= u * xc1;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < ROWS; ++j) {
    const int r = lane + 32 * j;
    if (r >= N) continue;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int q = q0 + h;
      if (q >= N) continue;
      const double g = q < N - 2 ? (h ? x1[j] : x0[j]) : 0.0;
      if (G) G[kb + (long long)r * N + q] = g;
      if (GT64) GT64[kb + (long long)q * N + r] = g;
      if (GT32) {
        const float hi = (float)g;
        GT32[kb + (long long)q * N + r] = make_float2(hi, (float)(g - (double)hi));
      }
    }
  }
}

// The same factorisation for matrices too large for shared memory (Nz of a
// few hundred): one CTA per matrix working in place in global memory (the
// matrix stays in L2 while its CTA factors it); the pivot column and the
// pivot row of each step are staged in shared memory for the rank-1 update.
__global__ void __launch_bounds__(512) smc_lu_medium_kernel(double* __restrict__ A, int* __restrict__ piv,
                                                            int* __restrict__ info, int N) {
  extern __shared__ double stage[];               // column c (N) + row c (N)
  double* colc = stage;
  double* rowc = stage + N;
  __shared__ double rv[32];
  __shared__ int ri[32];
  __shared__ int s_p;
  const int tid = threadIdx.x, nt = blockDim.x;
  double* a = A + (long long)blockIdx.x * N * N;
  int inf = 0;
  for (int c = 0; c < N; ++c) {
    double best = -1.0;
    int bi = N;
    for (int r = c + tid; r < N; r += nt) {
      double v = fabs(a[r + (long long)c * N]);
      if (v > best) { best = v; bi = r; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      double ov = __shfl_xor_sync(0xffffffffu, best, o);
      int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if ((tid & 31) == 0) { rv[tid >> 5] = best; ri[tid >> 5] = bi; }
    __syncthreads();
    if (tid == 0) {
      double b = rv[0];
      int p = ri[0];
      for (int w = 1; w < (nt >> 5); ++w)
        if (rv[w] > b || (rv[w] == b && ri[w] < p)) { b = rv[w]; p = ri[w]; }
      if (p >= N) p = c;
      s_p = p;
      piv[(long long)blockIdx.x * N + c] = p;
    }
    __syncthreads();
    const int p = s_p;
    if (p != c)
      for (int col = tid; col < N; col += nt) {
        double t = a[c + (long long)col * N];
        a[c + (long long)col * N] = a[p + (long long)col * N];
        a[p + (long long)col * N] = t;
      }
    __syncthreads();
    const double pv = a[c + (long long)c * N];
    if (pv != 0.0) {
      const double rinv = 1.0 / pv;
      for (int r = c + 1 + tid; r < N; r += nt) {
        const double l = a[r + (long long)c * N] * rinv;
        a[r + (long long)c * N] = l;
        colc[r] = l;
      }
    } else {
      if (!inf) inf = c + 1;
      for (int r = c + 1 + tid; r < N; r += nt) colc[r] = a[r + (long long)c * N];
    }
    for (int col = c + 1 + tid; col < N; col += nt) rowc[col] = a[c + (long long)col * N];
    __syncthreads();
    const int m = N - c - 1;
    for (int t = tid; t < m * m; t += nt) {
      const int r = c + 1 + t % m, col = c + 1 + t / m;
      a[r + (long long)col * N] -= colc[r] * rowc[col];
    }
    __syncthreads();
  }
  if (tid == 0 && info) info[blockIdx.x] = inf;
}


void lu_small_batched(const Ctx& c, double* A, int* piv, int* info, int N, int count) {
  size_t smem = (size_t)N * N * sizeof(double);
  if (smem > 200 * 1024) {
    smc_lu_medium_kernel<<<count, 512, 2 * N * sizeof(double), c.s>>>(A, piv, info, N);
    SMC_LAUNCH_CHECK(c);
    return;
  }
  allow_max_smem((const void*)smc_lu_small_kernel);
  smc_lu_small_kernel<<<count, 256, smem, c.s>>>(A, piv, info, N);
  SMC_LAUNCH_CHECK(c);
}

bool lu_green_batched(const Ctx& c, const double* A, double* LU, int* piv, double* G, double* GT64,
                      float2* GT32, int N, int count) {
  if (N > GL_MAXN) return false;
  if (A != LU)
    SMC_CUDA(cudaMemcpyAsync(LU, A, sizeof(double) * N * N * (size_t)count, cudaMemcpyDeviceToDevice, c.s));
  lu_small_batched(c, LU, piv, nullptr, N, count);
  const size_t smem = (size_t)(N * N + N) * sizeof(double);
  // columns per CTA: the CTAs that fit on the GPU at once share the count * N
  // columns (two per warp, 4..32 warps)
  const int fit = std::max(1, (int)((227 * 1024) / (smem + 1024)));
  const int slots = c.num_sms * fit;
  const int per = (int)((count * (long long)N + slots - 1) / slots);
  const int warps = std::min(32, std::max(4, (per + 1) / 2));
  const dim3 grd(count, (N + 2 * warps - 1) / (2 * warps));
  allow_max_smem((const void*)smc_green_lu_kernel);
  smc_green_lu_kernel<<<grd, 32 * warps, smem, c.s>>>(LU, piv, G, GT64, GT32, N);
  SMC_LAUNCH_CHECK(c);
  return true;
}

// In-place solve of one real LU factor (column-major, LAPACK ipiv) with a
// complex right-hand side held in shared memory.
__device__ void lu_real_solve_smem(const double* __restrict__ L, const int* __restrict__ pv,
                                   double2* xs, int N) {
  const int tid = threadIdx.x, nt = blockDim.x;
  if (tid == 0)
    for (int i = 0; i < N; ++i) {
      int p = pv[i];
      if (p != i) { double2 t = xs[i]; xs[i] = xs[p]; xs[p] = t; }
    }
  __syncthreads();
  for (int c = 0; c < N; ++c) {          // unit lower
    double2 xc = xs[c];
    for (int r = c + 1 + tid; r < N; r += nt) {
      double l = L[r + (long long)c * N];
      xs[r].x -= l * xc.x;
      xs[r].y -= l * xc.y;
    }
    __syncthreads();
  }
  for (int c = N - 1; c >= 0; --c) {     // upper
    if (tid == 0) {
      double u = L[c + (long long)c * N];
      xs[c].x /= u;
      xs[c].y /= u;
    }
    __syncthreads();
    double2 xc = xs[c];
    for (int r = tid; r < c; r += nt) {
      double u = L[r + (long long)c * N];
      xs[r].x -= u * xc.x;
      xs[r].y -= u * xc.y;
    }
    __syncthreads();
  }
}

// x_b = A_b^{-1} (alpha P b_b), complex right-hand side, real LU factor
__global__ void smc_lu_small_solve_kernel(const double* __restrict__ LU, const int* __restrict__ piv,
                                          long long lu_stride, const double2* __restrict__ b,
                                          double2* __restrict__ x, int N, double alpha,
                                          int zero_tau, const int* __restrict__ skip) {
  extern __shared__ double2 xs[];
  const int k = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  double2* xo = x + (long long)k * N;
  if (skip && skip[k]) {
    for (int i = tid; i < N; i += nt) xo[i] = make_double2(0.0, 0.0);
    return;
  }
  for (int i = tid; i < N; i += nt) {
    double2 v = b[(long long)k * N + i];
    if (zero_tau && i >= N - 2) v = make_double2(0.0, 0.0);
    xs[i] = make_double2(alpha * v.x, alpha * v.y);
  }
  __syncthreads();
  lu_real_solve_smem(LU + (long long)k * lu_stride, piv + (long long)k * N, xs, N);
  for (int i = tid; i < N; i += nt) xo[i] = xs[i];
}

// G_k[:, q] = A_k^{-1} e_q for q < N-2, 0 for the two tau columns
// (vv_stokes.py:281-296: G = solve(A, P)); one CTA per (k, q)
__global__ void smc_green_kernel(const double* __restrict__ LU, const int* __restrict__ piv,
                                 double* __restrict__ G, int N) {
  extern __shared__ double2 xs[];
  const int k = blockIdx.x, q = blockIdx.y, tid = threadIdx.x;
  double* Gk = G + (long long)k * N * N;
  if (q >= N - 2) {
    for (int p = tid; p < N; p += blockDim.x) Gk[(long long)p * N + q] = 0.0;
    return;
  }
  for (int i = tid; i < N; i += blockDim.x) xs[i] = make_double2(i == q ? 1.0 : 0.0, 0.0);
  __syncthreads();
  lu_real_solve_smem(LU + (long long)k * N * N, piv + (long long)k * N, xs, N);
  for (int p = tid; p < N; p += blockDim.x) Gk[(long long)p * N + q] = xs[p].x;
}

// The same columns, GREEN_COLS per 128-thread CTA and ZSPLIT lanes per
// column: lane s of a column's group updates the rows r = s (mod 4) at every
// substitution step, and the warp (8 groups) meets at __syncwarp before the
// next step reads the finished entry.  Every entry receives the updates of
// lu_real_solve_smem in the same order (the same values); the FP64 work
// spreads over 4x more warps than one thread per column, and no CTA-wide
// barrier is needed (the per-column CTAs above wait at 2N of them).
static constexpr int GREEN_COLS = 32;
static constexpr int GREEN_LD = GREEN_COLS + 1;       // padded row of the column block
static constexpr int GREEN_COLS_MAXN = 160;           // N x 33 doubles of shared memory <= 42 KB
__global__ void __launch_bounds__(GREEN_COLS * ZSPLIT) smc_green_cols_kernel(const double* __restrict__ LU,
                                                                            const int* __restrict__ piv,
                                                                            double* __restrict__ G, int N) {
  extern __shared__ double xcol[];       // row r of column cc at xcol[r * GREEN_LD + cc]
  const int k = blockIdx.x;
  const int cc = threadIdx.x / ZSPLIT, sub = threadIdx.x % ZSPLIT;
  const int q = blockIdx.y * GREEN_COLS + cc;
  const bool act = q < N - 2;            // the tau columns (and columns past N) are not solved
  const double* L = LU + (long long)k * N * N;
  const int* pv = piv + (long long)k * N;
  double* x = xcol + cc;
  // every lane runs every step loop (the __syncwarp calls need the whole warp)
  if (act)
    for (int i = sub; i < N; i += ZSPLIT) x[i * GREEN_LD] = (i == q) ? 1.0 : 0.0;
  __syncwarp();
  if (act && sub == 0)
    for (int i = 0; i < N; ++i) {
      const int p = pv[i];
      if (p != i) {
        const double t = x[i * GREEN_LD];
        x[i * GREEN_LD] = x[p * GREEN_LD];
        x[p * GREEN_LD] = t;
      }
    }
  __syncwarp();
  for (int c = 0; c < N; ++c) {          // unit lower
    if (act) {
      const double xc = x[c * GREEN_LD];
      const double* Lc = L + (long long)c * N;
      for (int r = c + 1 + ((sub - c - 1) & (ZSPLIT - 1)); r < N; r += ZSPLIT)
        x[r * GREEN_LD] -= Lc[r] * xc;
    }
    __syncwarp();
  }
  for (int c = N - 1; c >= 0; --c) {     // upper
    const double* Lc = L + (long long)c * N;
    if (act && sub == (c & (ZSPLIT - 1))) x[c * GREEN_LD] /= Lc[c];
    __syncwarp();
    if (act) {
      const double xc = x[c * GREEN_LD];
      for (int r = sub; r < c; r += ZSPLIT) x[r * GREEN_LD] -= Lc[r] * xc;
    }
    __syncwarp();
  }
  if (q < N) {
    double* Gk = G + (long long)k * N * N;
    for (int p = sub; p < N; p += ZSPLIT) Gk[(long long)p * N + q] = act ? x[p * GREEN_LD] : 0.0;
  }
}

void green_from_lu(const Ctx& c, const double* LUcm, const int* piv, double* G, int N, int Nk) {
  if (N <= GREEN_COLS_MAXN) {
    dim3 grd(Nk, (N + GREEN_COLS - 1) / GREEN_COLS);
    smc_green_cols_kernel<<<grd, GREEN_COLS * ZSPLIT, (size_t)N * GREEN_LD * sizeof(double), c.s>>>(
        LUcm, piv, G, N);
  } else {
    dim3 grd(Nk, N);
    smc_green_kernel<<<grd, 128, N * sizeof(double2), c.s>>>(LUcm, piv, G, N);
  }
  SMC_LAUNCH_CHECK(c);
}

void lu_small_solve(const Ctx& c, const double* LU, const int* piv, long long lu_stride,
                    const double2* b, double2* x, int N, int count, double alpha, int zero_tau,
                    const int* skip_mask) {
  size_t smem = (size_t)N * sizeof(double2);
  smc_lu_small_solve_kernel<<<count, 128, smem, c.s>>>(LU, piv, lu_stride, b, x, N, alpha,
                                                       zero_tau, skip_mask);
  SMC_LAUNCH_CHECK(c);
}

// ======================================================== dense complex LU
static constexpr int ZNB = 32;     // panel width
static constexpr int ZROWCHUNK = 32;

// rows of the column range [r_lo, n) owned by CTA b: chunks of 32 rows dealt
// round-robin over the grid (chunk ch belongs to CTA ch mod G).  Inside the
// CTA, warp w takes the CTA's chunks w, w + nwarps, ...; lane l handles row
// 32 ch + l, so a warp's loads of one column are one coalesced 512-byte line
// and a given row is always handled by the same thread during a panel.
// The body runs once per (chunk, lane); `continue` skips that row.
#define SMC_FOR_OWNED_ROW(r, r_lo, n, b, G, warp, nwarps, lane)                          \
  for (int ch_ = ((r_lo) / ZROWCHUNK + (((b) - ((r_lo) / ZROWCHUNK) % (G)) + (G)) % (G)) + \
                 (warp) * (G);                                                           \
       ch_ * ZROWCHUNK < (n); ch_ += (G) * (nwarps))                                     \
    for (int r = ch_ * ZROWCHUNK + (lane), once_ = 1; once_; once_ = 0)                  \
      if (r >= (r_lo) && r < (n))

__device__ __forceinline__ void argmax_merge(double& v, int& i, double ov, int oi) {
  if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; }
}

// Panel factorisation of columns [p0, p0+nbp): cooperative, one CTA per SM,
// ONE grid barrier per column.  Rows are not swapped during the panel: the
// pivot row of column c stays at its physical position p and is marked done
// (excluded from later pivot searches and updates), which removes the race a
// physical swap would have with the other CTAs' reads.  After the last
// column the sequence of pivot rows is converted into LAPACK's sequential
// interchanges ipiv, and laswp applies them to every column (panel included):
// the elimination arithmetic of each row does not depend on where it sits, so
// the result is the LAPACK layout.  Candidate pivots are double-buffered
// (part[(c & 1)]) so a fast CTA never overwrites a slot a slow one is reading.
__global__ void smc_zlu_panel_kernel(double2* __restrict__ A, int n, int p0, int nbp,
                                     int* __restrict__ piv, double* __restrict__ part,
                                     int* __restrict__ done, int* __restrict__ pv) {
  cg::grid_group grid = cg::this_grid();
  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  __shared__ double rv[32];
  __shared__ int ri[32];
  __shared__ int s_p;
  __shared__ double2 prow[ZNB];
  // mark owned rows not done; local argmax of the first column
  double best = -1.0;
  int bi = n;
  const int nwarps = nt >> 5;
  SMC_FOR_OWNED_ROW(r, p0, n, b, G, warp, nwarps, lane) {
    done[r] = 0;
    double v = cabs1(A[r + (long long)p0 * n]);
    if (v != v) v = INFINITY;
    argmax_merge(best, bi, v, r);
  }
  for (int t = 0; t < nbp; ++t) {
    const int c = p0 + t;
    double* pw = part + (size_t)(t & 1) * 2 * G;
    for (int o = 16; o > 0; o >>= 1)
      argmax_merge(best, bi, __shfl_xor_sync(0xffffffffu, best, o), __shfl_xor_sync(0xffffffffu, bi, o));
    if (lane == 0) { rv[warp] = best; ri[warp] = bi; }
    __syncthreads();
    if (tid == 0) {
      double v = rv[0];
      int i = ri[0];
      for (int w = 1; w < (nt >> 5); ++w) argmax_merge(v, i, rv[w], ri[w]);
      pw[2 * b] = v;
      pw[2 * b + 1] = (double)i;
    }
    grid.sync();
    // global pivot, warp-parallel over the G candidates
    if (warp == 0) {
      double v = -1.0;
      int i = n;
      for (int g = lane; g < G; g += 32) argmax_merge(v, i, pw[2 * g], (int)pw[2 * g + 1]);
      for (int o = 16; o > 0; o >>= 1)
        argmax_merge(v, i, __shfl_xor_sync(0xffffffffu, v, o), __shfl_xor_sync(0xffffffffu, i, o));
      if (lane == 0) {
        if (i >= n) i = c;          // all-zero or empty column: keep the diagonal
        s_p = i;
      }
    }
    __syncthreads();
    const int p = s_p;
    if (b == 0 && tid == 0) pv[t] = p;
    for (int col = c + tid; col < p0 + nbp; col += nt) prow[col - c] = A[p + (long long)col * n];
    __syncthreads();
    const double2 pivv = prow[0];
    const bool nz = (pivv.x != 0.0 || pivv.y != 0.0);
    const double2 rinv = nz ? cdiv(make_double2(1.0, 0.0), pivv) : make_double2(0.0, 0.0);
    const int ncols = p0 + nbp - c - 1;
    best = -1.0;
    bi = n;
    SMC_FOR_OWNED_ROW(r, p0, n, b, G, warp, nwarps, lane) {
      if (r == p) { done[r] = 1; continue; }
      if (done[r]) continue;
      double2* Ar = A + r + (long long)c * n;
      double2 l = Ar[0];
      if (nz) l = cmul(l, rinv);
      Ar[0] = l;
      // the row's remaining panel entries, eight loads in flight before their
      // stores (a store could alias a later load as far as the compiler
      // knows, which would otherwise serialise the loop on memory latency)
      double2 next = make_double2(0.0, 0.0);   // updated entry of column c+1
      int j = 1;
      for (; j + 7 <= ncols; j += 8) {
        double2 e[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) e[q] = Ar[(long long)(j + q) * n];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          e[q] = csub(e[q], cmul(l, prow[j + q]));
          Ar[(long long)(j + q) * n] = e[q];
        }
        if (j == 1) next = e[0];
      }
      for (; j <= ncols; ++j) {
        double2 e = csub(Ar[(long long)j * n], cmul(l, prow[j]));
        Ar[(long long)j * n] = e;
        if (j == 1) next = e;
      }
      if (t + 1 < nbp) {
        double v = cabs1(next);
        if (v != v) v = INFINITY;
        argmax_merge(best, bi, v, r);
      }
    }
    __syncthreads();
  }
  // pivot rows (physical, unswapped) -> LAPACK sequential interchanges
  if (b == 0 && tid == 0) {
    int rowid[2 * ZNB], posn[2 * ZNB];   // tracked rows and their current positions
    int nt2 = 0;
    for (int t = 0; t < nbp; ++t) {
      const int q = p0 + t, r = pv[t];
      int pr = r;                    // current position of row r
      for (int k = 0; k < nt2; ++k) if (rowid[k] == r) { pr = posn[k]; break; }
      int rq = q;                    // row currently at position q
      for (int k = 0; k < nt2; ++k) if (posn[k] == q) { rq = rowid[k]; break; }
      piv[q] = pr;
      // swap: row r -> q, row rq -> pr
      bool fr = false, fq = false;
      for (int k = 0; k < nt2; ++k) {
        if (rowid[k] == r) { posn[k] = q; fr = true; }
        else if (rowid[k] == rq) { posn[k] = pr; fq = true; }
      }
      if (!fr && nt2 < 2 * ZNB) { rowid[nt2] = r; posn[nt2] = q; ++nt2; }
      if (!fq && rq != r && nt2 < 2 * ZNB) { rowid[nt2] = rq; posn[nt2] = pr; ++nt2; }
    }
    // the same interchanges as one gather: position posn[k] receives the
    // original row rowid[k] (rows that did not move are left out)
    int* gl = pv + ZNB;
    int m = 0;
    for (int k = 0; k < nt2; ++k)
      if (rowid[k] != posn[k]) { gl[1 + m] = rowid[k]; gl[1 + 2 * ZNB + m] = posn[k]; ++m; }
    gl[0] = m;
  }
}

// row interchanges of panel [p0, p0+nbp) applied to every column, as the
// gather the panel kernel left in gl = {m, src[2 ZNB], dst[2 ZNB]}: one warp
// per column, each lane moving up to two rows; all loads of a column precede
// its stores.
static constexpr int LASWP_WARPS = 8;
__global__ void __launch_bounds__(32 * LASWP_WARPS) smc_zlu_laswp_kernel(double2* __restrict__ A, int n,
                                                                         const int* __restrict__ gl) {
  __shared__ int s_src[2 * ZNB], s_dst[2 * ZNB];
  __shared__ int s_m;
  if (threadIdx.x == 0) s_m = min(gl[0], 2 * ZNB);
  __syncthreads();
  const int m = s_m;
  for (int t = threadIdx.x; t < m; t += blockDim.x) { s_src[t] = gl[1 + t]; s_dst[t] = gl[1 + 2 * ZNB + t]; }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int col = blockIdx.x * LASWP_WARPS + (threadIdx.x >> 5);
  if (col >= n) return;
  double2* Ac = A + (long long)col * n;
  double2 v0 = make_double2(0.0, 0.0), v1 = v0;
  if (lane < m) v0 = Ac[s_src[lane]];
  if (lane + 32 < m) v1 = Ac[s_src[lane + 32]];
  __syncwarp();
  if (lane < m) Ac[s_dst[lane]] = v0;
  if (lane + 32 < m) Ac[s_dst[lane + 32]] = v1;
}

// U12 = L11^{-1} A12 (unit lower L11 of the panel), one warp per column:
// lane i holds entry i of the column; forward substitution broadcasts the
// finished entry c with a shuffle and every lane below it subtracts its
// multiple.  Loads and stores of a column are one coalesced line.
static constexpr int TRSM_WARPS = 8;
__global__ void __launch_bounds__(32 * TRSM_WARPS) smc_zlu_trsm_kernel(double2* __restrict__ A, int n,
                                                                       int p0, int nbp) {
  __shared__ double2 L[ZNB * ZNB];     // L[r + c*ZNB]
  for (int t = threadIdx.x; t < nbp * nbp; t += blockDim.x) {
    int r = t % nbp, c = t / nbp;
    L[r + c * ZNB] = A[(p0 + r) + (long long)(p0 + c) * n];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int col = p0 + nbp + blockIdx.x * TRSM_WARPS + (threadIdx.x >> 5);
  if (col >= n) return;              // uniform per warp
  double2* Ac = A + (long long)col * n + p0;
  double2 x = lane < nbp ? Ac[lane] : make_double2(0.0, 0.0);
  for (int c = 0; c + 1 < nbp; ++c) {
    double2 xc;
    xc.x = __shfl_sync(0xffffffffu, x.x, c);
    xc.y = __shfl_sync(0xffffffffu, x.y, c);
    if (lane > c && lane < nbp) x = csub(x, cmul(L[lane + c * ZNB], xc));
  }
  if (lane < nbp) Ac[lane] = x;
}

// A22 -= L21 U12 : 64x64 output tile per CTA, 4x4 complex outputs per thread
static constexpr int GT = 64;
__global__ void __launch_bounds__(256) smc_zlu_gemm_kernel(double2* __restrict__ A, int n, int p0, int nbp) {
  extern __shared__ double2 sm[];
  double2* Ls = sm;                    // [nbp][GT] : Ls[kk*GT + r]
  double2* Us = sm + ZNB * GT;         // [nbp][GT] : Us[kk*GT + c]
  const int r0 = p0 + nbp + blockIdx.y * GT;
  const int c0 = p0 + nbp + blockIdx.x * GT;
  const int tid = threadIdx.x;
  for (int t = tid; t < nbp * GT; t += 256) {
    int r = t % GT, kk = t / GT;
    int gr = r0 + r;
    Ls[kk * GT + r] = (gr < n) ? A[gr + (long long)(p0 + kk) * n] : make_double2(0.0, 0.0);
  }
  for (int t = tid; t < nbp * GT; t += 256) {
    int k2 = t % nbp, cc = t / nbp;
    int gc = c0 + cc;
    Us[k2 * GT + cc] = (gc < n) ? A[(p0 + k2) + (long long)gc * n] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  const int tr = (tid % 16) * 4, tc = (tid / 16) * 4;
  double2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_double2(0.0, 0.0);
  for (int kk = 0; kk < nbp; ++kk) {
    double2 l[4], u[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) l[i] = Ls[kk * GT + tr + i];
#pragma unroll
    for (int j = 0; j < 4; ++j) u[j] = Us[kk * GT + tc + j];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        acc[i][j].x += l[i].x * u[j].x - l[i].y * u[j].y;
        acc[i][j].y += l[i].x * u[j].y + l[i].y * u[j].x;
      }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    int gc = c0 + tc + j;
    if (gc >= n) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int gr = r0 + tr + i;
      if (gr >= n) continue;
      double2* e = &A[gr + (long long)gc * n];
      *e = csub(*e, acc[i][j]);
    }
  }
}

void zlu_dense(const Ctx& c, double2* A, int* piv, int n, double2* work, void* tcwork,
               int* tcerr) {
  const size_t gsm = (size_t)2 * ZNB * GT * sizeof(double2);
  allow_max_smem((const void*)smc_zlu_gemm_kernel);
  int G = c.num_sms;
  int maxb = 0;
  SMC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, smc_zlu_panel_kernel, 256, 0));
  if (maxb < 1) throw std::runtime_error("zlu_dense: panel kernel cannot be co-resident");
  double* part = reinterpret_cast<double*>(work);                 // 4 G doubles
  int* done = reinterpret_cast<int*>(part + 4 * G + 64);           // n ints
  int* pv = done + n + 64;        // ZNB pivot rows, then the gather list (1 + 4 ZNB ints)
  for (int p0 = 0; p0 < n; p0 += ZNB) {
    int nbp = std::min(ZNB, n - p0);
    void* args[] = {&A, &n, &p0, &nbp, &piv, &part, &done, &pv};
    {
      CoopGuard guard(c.s);
      SMC_CUDA(cudaLaunchCooperativeKernel((void*)smc_zlu_panel_kernel, dim3(G), dim3(256), args, 0, c.s));
      SMC_LAUNCH_CHECK(c);
    }
    smc_zlu_laswp_kernel<<<ceil_div(n, LASWP_WARPS), 32 * LASWP_WARPS, 0, c.s>>>(A, n, pv + ZNB);
    SMC_LAUNCH_CHECK(c);
    int rest = n - p0 - nbp;
    if (rest > 0) {
      smc_zlu_trsm_kernel<<<ceil_div(rest, TRSM_WARPS), 32 * TRSM_WARPS, 0, c.s>>>(A, n, p0, nbp);
      SMC_LAUNCH_CHECK(c);
      if (tcwork) {
        tclu_update(c, A, n, p0, nbp, tcwork, tcerr);
      } else {
        dim3 g(ceil_div(rest, GT), ceil_div(rest, GT));
        smc_zlu_gemm_kernel<<<g, 256, gsm, c.s>>>(A, n, p0, nbp);
        SMC_LAUNCH_CHECK(c);
      }
    }
  }
}

// ================================================== dense triangular solve
static constexpr int SB = 64;      // diagonal block of the solve

// Inverses of the SB x SB diagonal blocks of L (unit lower) and U (upper),
// column-major, computed once per factorisation: blockIdx.x = block,
// blockIdx.y = 0 (L) / 1 (U).  Thread c forms column c of the inverse.
__global__ void smc_zlu_diag_inv_kernel(const double2* __restrict__ LU, int n,
                                        double2* __restrict__ invL, double2* __restrict__ invU) {
  extern __shared__ double2 sm[];
  double2* Bk = sm;               // SB*SB block
  double2* X = sm + SB * SB;      // SB*SB inverse
  const int bk = blockIdx.x, upper = blockIdx.y;
  const int r0 = bk * SB, m = min(SB, n - r0);
  for (int t = threadIdx.x; t < SB * SB; t += blockDim.x) {
    int r = t % SB, c = t / SB;
    Bk[t] = (r < m && c < m) ? LU[(r0 + r) + (long long)(r0 + c) * n]
                             : make_double2((r == c) ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  const int c = threadIdx.x;
  if (c < SB) {
    double2* x = X + c * SB;
    if (!upper) {
      for (int r = 0; r < SB; ++r) x[r] = make_double2(r == c ? 1.0 : 0.0, 0.0);
      for (int r = c + 1; r < SB; ++r) {
        double2 acc = x[r];
        for (int j = c; j < r; ++j) acc = csub(acc, cmul(Bk[r + j * SB], x[j]));
        x[r] = acc;
      }
    } else {
      for (int r = 0; r < SB; ++r) x[r] = make_double2(0.0, 0.0);
      for (int r = c; r >= 0; --r) {
        double2 acc = make_double2(r == c ? 1.0 : 0.0, 0.0);
        for (int j = r + 1; j <= c; ++j) acc = csub(acc, cmul(Bk[r + j * SB], x[j]));
        x[r] = cdiv(acc, Bk[r + r * SB]);
      }
    }
  }
  __syncthreads();
  double2* dst = (upper ? invU : invL) + (long long)bk * SB * SB;
  for (int t = threadIdx.x; t < SB * SB; t += blockDim.x) dst[t] = X[t];
}

__device__ __forceinline__ int first_owned_chunk(int row_lo, int b, int G) {
  int c0 = row_lo / 32;
  return c0 + ((b - c0 % G) % G + G) % G;
}

// One block step of the solve.  Every CTA forms x_blk = inv(D_bk) w[r0:r1]
// (a 64 x 64 GEMV, redundant across CTAs so no barrier is needed inside the
// step); the block's owner writes x_blk to `dst`; each CTA then updates the
// rows it owns (32-row chunks dealt round-robin) below (forward) or above
// (backward) the block.  The forward sweep updates `x` in place and writes
// solved blocks to `y`, the backward sweep updates `y` and writes to `x`,
// so a block is never written while another CTA may still be reading it.
template <bool LOWER>
__device__ void smc_trsv_block(const double2* __restrict__ LU, const double2* __restrict__ inv,
                               double2* __restrict__ work, double2* __restrict__ dst, int n,
                               int bk, double2* win, double2* xb, double2 (*red)[32]) {
  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int r0 = bk * SB, r1 = min(n, r0 + SB), m = r1 - r0;
  const int lo = LOWER ? r1 : 0, hi = LOWER ? n : r0;
  const bool owner = (b == bk % G);
  const bool has_rows = first_owned_chunk(lo, b, G) * 32 < hi;
  if (!owner && !has_rows) return;
  if (tid < SB) win[tid] = (tid < m) ? work[r0 + tid] : make_double2(0.0, 0.0);
  __syncthreads();
  {
    // xb[i] = sum_j inv[i + j*SB] win[j]: 4 threads per row, 16 terms each
    const int i = tid & 63, qd = tid >> 6;
    const double2* Ib = inv + (long long)bk * SB * SB;
    double2 acc = make_double2(0.0, 0.0);
    for (int j = qd * 16; j < qd * 16 + 16; ++j) acc = cadd(acc, cmul(Ib[i + j * SB], win[j]));
    double2* rf = &red[0][0];          // viewed as [4][64]
    rf[qd * 64 + i] = acc;
    __syncthreads();
    if (tid < 64) xb[tid] = cadd(cadd(rf[tid], rf[64 + tid]), cadd(rf[128 + tid], rf[192 + tid]));
    __syncthreads();
  }
  if (owner)
    for (int i = tid; i < m; i += 256) dst[r0 + i] = xb[i];
  for (int ch = first_owned_chunk(lo, b, G); ch * 32 < hi; ch += G) {
    int r = ch * 32 + lane;
    bool act = (r >= lo && r < hi);
    double2 acc = make_double2(0.0, 0.0);
    if (act)
      for (int cc = warp; cc < m; cc += 8) acc = cadd(acc, cmul(LU[r + (long long)(r0 + cc) * n], xb[cc]));
    red[warp][lane] = acc;
    __syncthreads();
    if (warp == 0 && act) {
      double2 s = red[0][lane];
      for (int w = 1; w < 8; ++w) s = cadd(s, red[w][lane]);
      work[r] = csub(work[r], s);
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) smc_zlu_solve_kernel(const double2* __restrict__ LU,
                                                           const double2* __restrict__ invL,
                                                           const double2* __restrict__ invU,
                                                           const int* __restrict__ perm,
                                                           const double2* __restrict__ bvec,
                                                           double2* __restrict__ x,
                                                           double2* __restrict__ y, int n) {
  cg::grid_group grid = cg::this_grid();
  __shared__ double2 win[SB];
  __shared__ double2 xb[SB];
  __shared__ double2 red[8][32];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = bvec[perm[i]];
  grid.sync();
  const int nblk = (n + SB - 1) / SB;
  for (int bk = 0; bk < nblk; ++bk) {
    smc_trsv_block<true>(LU, invL, x, y, n, bk, win, xb, red);
    grid.sync();
  }
  for (int bk = nblk - 1; bk >= 0; --bk) {
    smc_trsv_block<false>(LU, invU, y, x, n, bk, win, xb, red);
    grid.sync();
  }
}

void zlu_diag_inverses(const Ctx& c, const double2* LU, int n, double2* invL, double2* invU) {
  const int nblk = (n + SB - 1) / SB;
  const size_t sm = (size_t)2 * SB * SB * sizeof(double2);
  allow_max_smem((const void*)smc_zlu_diag_inv_kernel);
  smc_zlu_diag_inv_kernel<<<dim3(nblk, 2), 64, sm, c.s>>>(LU, n, invL, invU);
  SMC_LAUNCH_CHECK(c);
}

void zlu_dense_solve(const Ctx& c, const double2* LU, const double2* invL, const double2* invU,
                     const int* perm, const double2* b, double2* x, int n, double2* work) {
  int G = c.num_sms;
  int maxb = 0;
  SMC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, smc_zlu_solve_kernel, 256, 0));
  if (maxb < 1) throw std::runtime_error("zlu_dense_solve: kernel cannot be co-resident");
  double2* y = work;
  void* args[] = {(void*)&LU, (void*)&invL, (void*)&invU, (void*)&perm, (void*)&b,
                  (void*)&x, (void*)&y, (void*)&n};
  CoopGuard guard(c.s);
  SMC_CUDA(cudaLaunchCooperativeKernel((void*)smc_zlu_solve_kernel, dim3(G), dim3(256), args, 0, c.s));
  SMC_LAUNCH_CHECK(c);
}

}  // namespace smc
