// Persistent Krylov engine of the fast form: one cooperative launch runs a
// whole right-preconditioned FGMRES solve (core/krylov_fgmres.py:60-179) on
// the device -- preconditioner, operator, CGS2 Arnoldi and the Givens
// least-squares update -- with no host round trip per iteration.
//
// Operators: the fused Schur matvec (stokes/lagged_stokes.py:202-220) or the
// fused temperature matvec (implicit_theta.py:354-383).  Everything of the
// Krylov process -- basis vectors, dot products, Hessenberg matrix, Givens
// rotations -- is carried in the working precision T: float for the inner
// solves of the mixed form (which only have to reach a relative residual of
// about 1e-4 before the FP64 refinement takes over), double for a solve in
// FP64.  Only the right-hand side b and the solution x are FP64.
//
// Work decomposition.  Both operators have the shape
//     per-k z-contraction -> per-z-point x-convolution -> per-k z-epilogue,
// and the block preconditioner acts on one Fourier row k at a time.  The grid
// is split into Nk groups of R = G / Nk CTAs; the CTAs of group k each build
// the whole row k of the next basis vector and of its preconditioned vector
// (redundantly -- a row is N values), then each contracts its own slice of
// output rows.  So one Arnoldi step is four phases separated by grid
// barriers:
//   NEXT   v_{j} = (w' - V h2) / h, z_j = M v_j, z-contraction      (per k)
//   XCONV  x-direction convolution                          (per z-point)
//   POST   w = z-epilogue, first-pass dots V^H w            (per k, rows)
//   UPDATE w' = w - V h1, second-pass dots V^H w', ||w'||^2 (per k, rows)
// The norm of w'' = w' - V h2 follows from ||w''||^2 = ||w'||^2 - ||h2||^2;
// when that difference cancels badly an exact norm is taken with one extra
// barrier.  Every CTA reduces the per-CTA dot partials in the same order and
// runs the Givens update itself, so all CTAs hold identical coefficients and
// take identical branches.
//
// Uniform control: every branch that decides how many grid barriers a CTA
// executes depends only on values every CTA computes identically from the
// same data after the same barrier, and every loop is bounded by the restart
// length and the iteration budget, so all CTAs execute the same sequence of
// barriers.
#include <cooperative_groups.h>

#include <type_traits>

#include "smc_internal.cuh"
#include "smc_engine.cuh"
#include "smc_fft.cuh"

namespace cg = cooperative_groups;

namespace smc {

template <class T> struct CT2;
template <> struct CT2<double> { using type = double2; };
template <> struct CT2<float> { using type = float2; };
template <class T> using Cx = typename CT2<T>::type;

static constexpr int ENG_THREADS = 256;
static constexpr int ENG_WARPS = ENG_THREADS / 32;
static constexpr int ENG_MAXM = 100;     // restart + 1
static constexpr int RCH = 64;           // output rows per GEMV chunk

struct EngCtx {
  int G, b, tid, lane, warp, gw, nw;   // grid size, block, thread, lane, warp, global warp, #warps
  int R, ntask;                        // CTAs per Fourier row, row tasks
};

#define SMC_PHASE_NAMES(P)                                                                   \
  {P ".start", P ".xconv", P ".xconv_wait", P ".post", P ".post_wait", P ".update_reduce",      \
   P ".update", P ".update_wait", P ".exact_norm", P ".next_reduce", P ".givens", P ".combine", \
   P ".precond", P ".contract", P ".next_wait", P ".lsq", P ".resid", P ".refine_xupdate",     \
   P ".refine_contract", P ".refine_xconv", P ".refine_post", P ".refine_norm", P ".total_cycles", \
   P ".total_ns"}
const char* const engine_phase_names[2][ENGINE_PHASES] = {SMC_PHASE_NAMES("engine_stokes"),
                                                          SMC_PHASE_NAMES("engine_theta")};
#undef SMC_PHASE_NAMES

// phase timer of CTA 0 / thread 0: cycles since the previous mark go to slot
__device__ __forceinline__ long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return (long long)t;
}

struct PhaseClock {
  long long* acc;
  long long last, c0, ns0;
  __device__ void init(long long* a, const EngCtx& e) {
    acc = (a && e.b == 0 && e.tid == 0) ? a : nullptr;
    last = c0 = clock64();
    ns0 = acc ? global_ns() : 0;
  }
  // the launch's totals (call once, at the end)
  __device__ void finish() {
    if (acc) {
      acc[EP_TOTAL_CYCLES] += clock64() - c0;
      acc[EP_TOTAL_NS] += global_ns() - ns0;
    }
  }
  __device__ void mark(int slot) {
    if (acc) {
      const long long t = clock64();
      acc[slot] += t - last;
      last = t;
    }
  }
};

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ------------------------------------------------- complex arithmetic in T
template <class T>
__device__ __forceinline__ Cx<T> mk2(T a, T b) {
  Cx<T> r;
  r.x = a;
  r.y = b;
  return r;
}
template <class T> __device__ __forceinline__ Cx<T> x_add(Cx<T> a, Cx<T> b) { return mk2<T>(a.x + b.x, a.y + b.y); }
template <class T> __device__ __forceinline__ Cx<T> x_sub(Cx<T> a, Cx<T> b) { return mk2<T>(a.x - b.x, a.y - b.y); }
template <class T> __device__ __forceinline__ Cx<T> x_mul(Cx<T> a, Cx<T> b) {
  return mk2<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class T> __device__ __forceinline__ Cx<T> x_scale(Cx<T> a, T s) { return mk2<T>(a.x * s, a.y * s); }
template <class T> __device__ __forceinline__ Cx<T> x_conj(Cx<T> a) { return mk2<T>(a.x, -a.y); }
// a / b, Smith's scaling
template <class T> __device__ __forceinline__ Cx<T> x_div(Cx<T> a, Cx<T> b) {
  if (fabs(b.x) >= fabs(b.y)) {
    const T r = b.y / b.x, d = b.x + b.y * r;
    return mk2<T>((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  }
  const T r = b.x / b.y, d = b.y + b.x * r;
  return mk2<T>((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
template <class T> __device__ __forceinline__ T x_abs(Cx<T> a) { return hypot(a.x, a.y); }

// per-CTA shared-memory rows of the per-k phases (carved from dynamic smem;
// the x-convolution phases reuse the same bytes from offset 0)
template <class T>
struct EngSmem {
  using C = Cx<T>;
  C* v;       // N   row being formed (basis row / epilogue input)
  C* w;       // N   epilogue outputs / updated rows of the task
  C* z;       // N   preconditioned row (contraction input)
  C* aux;     // max(4 Mz, N) epilogue vectors
  C* out;     // 4 RCH GEMV results
  void* red;  // warp partials
};

__host__ __device__ inline size_t eng_align(size_t b) { return (b + 255) & ~(size_t)255; }

template <class T>
__host__ __device__ inline size_t eng_red_bytes() {
  using C = Cx<T>;
  const size_t a = (size_t)ENG_WARPS * 4 * RCH * sizeof(C);      // 4-matrix GEMV partials
  const size_t b = (size_t)ENG_WARPS * RCH * 16;                  // double-float / FP64 partials
  const size_t c = (size_t)ENG_WARPS * RCH * 48;                  // mixed z-contraction (T = float)
  const size_t m = a > b ? a : b;
  return m > c ? m : c;
}

template <class T>
__host__ __device__ inline size_t eng_rows_bytes(int N, int Mz) {
  using C = Cx<T>;
  const size_t aux = (size_t)(4 * Mz > N ? 4 * Mz : N);
  return eng_align((size_t)N * sizeof(C)) * 3 + eng_align(aux * sizeof(C)) +
         eng_align(4 * RCH * sizeof(C)) + eng_align(eng_red_bytes<T>());
}

template <class T>
__device__ EngSmem<T> eng_carve(unsigned char* base, int N, int Mz) {
  using C = Cx<T>;
  EngSmem<T> S;
  size_t o = 0;
  const int aux = 4 * Mz > N ? 4 * Mz : N;
  S.v = reinterpret_cast<C*>(base + o); o += eng_align((size_t)N * sizeof(C));
  S.w = reinterpret_cast<C*>(base + o); o += eng_align((size_t)N * sizeof(C));
  S.z = reinterpret_cast<C*>(base + o); o += eng_align((size_t)N * sizeof(C));
  S.aux = reinterpret_cast<C*>(base + o); o += eng_align((size_t)aux * sizeof(C));
  S.out = reinterpret_cast<C*>(base + o); o += eng_align(4 * RCH * sizeof(C));
  S.red = base + o;
  return S;
}

// ----------------------------------------------------------- row helpers
// out[m][r] = sum_c At[m][c ld + r0 + r] x[m][c] for r < nr <= RCH, m < NM:
// lanes over output rows (coalesced in the transposed layout), warps over
// columns, warp partials summed in a fixed order.  Ends with __syncthreads.
template <class T, int NM>
struct GemvArgs {
  const T* a[NM];
  const Cx<T>* x[NM];
};

template <class T, int NM>
__device__ void tgemv_chunk(const GemvArgs<T, NM>& g, long long ld, int r0, int nr, int ncol,
                            EngSmem<T>& S, const EngCtx& e) {
  using C = Cx<T>;
  C* red = reinterpret_cast<C*>(S.red);
  for (int rc = 0; rc < nr; rc += 32) {
    const int r = rc + e.lane;
    T ar[NM], ai[NM];
#pragma unroll
    for (int m = 0; m < NM; ++m) { ar[m] = (T)0; ai[m] = (T)0; }
    if (r < nr) {
#pragma unroll 4
      for (int c = e.warp; c < ncol; c += ENG_WARPS) {
#pragma unroll
        for (int m = 0; m < NM; ++m) {
          const T a = g.a[m][(long long)c * ld + r0 + r];
          const C x = g.x[m][c];
          ar[m] += a * x.x;
          ai[m] += a * x.y;
        }
      }
    }
#pragma unroll
    for (int m = 0; m < NM; ++m) red[(e.warp * NM + m) * RCH + r] = mk2<T>(ar[m], ai[m]);
  }
  __syncthreads();
  for (int idx = e.tid; idx < NM * nr; idx += blockDim.x) {
    const int m = idx / nr, r = idx - m * nr;
    T sr = (T)0, si = (T)0;
    for (int w = 0; w < ENG_WARPS; ++w) {
      const C q = red[(w * NM + m) * RCH + r];
      sr += q.x;
      si += q.y;
    }
    S.out[m * RCH + r] = mk2<T>(sr, si);
  }
  __syncthreads();
}

// y[r] = (base[off + r] - sum_{i<mm} c_i V_i[off + r]) * scale for r < nr;
// warps over i, lanes over r.  Results go to the shared row y and/or to
// global gout[off + r].  Ends with __syncthreads.
template <class T>
__device__ void combine_rows(const Cx<T>* base, const Cx<T>* V, long long n, long long off, int nr,
                             const Cx<T>* c, int mm, T scale, Cx<T>* y, Cx<T>* gout,
                             EngSmem<T>& S, const EngCtx& e) {
  using C = Cx<T>;
  C* red = reinterpret_cast<C*>(S.red);
  for (int r0 = 0; r0 < nr; r0 += RCH) {
    const int cnt = min(RCH, nr - r0);
    for (int rc = 0; rc < cnt; rc += 32) {
      const int r = rc + e.lane;
      T sr = (T)0, si = (T)0;
      if (r < cnt) {
#pragma unroll 4
        for (int i = e.warp; i < mm; i += ENG_WARPS) {
          const C v = V[(long long)i * n + off + r0 + r];
          const C ci = c[i];
          sr += ci.x * v.x - ci.y * v.y;
          si += ci.x * v.y + ci.y * v.x;
        }
      }
      red[e.warp * RCH + r] = mk2<T>(sr, si);
    }
    __syncthreads();
    for (int r = e.tid; r < cnt; r += blockDim.x) {
      T sr = (T)0, si = (T)0;
      for (int w = 0; w < ENG_WARPS; ++w) {
        sr += red[w * RCH + r].x;
        si += red[w * RCH + r].y;
      }
      const C bv = base ? base[off + r0 + r] : mk2<T>((T)0, (T)0);
      const C o = mk2<T>((bv.x - sr) * scale, (bv.y - si) * scale);
      if (y) y[r0 + r] = o;
      if (gout) gout[off + r0 + r] = o;
    }
    __syncthreads();
  }
}

// acc[i] += sum_{r<nr} conj(V_i[off + r]) y[r] for i < mm: warps over i in
// batches of four (independent loads), lanes over r
template <class T>
__device__ void dots_acc(const Cx<T>* V, long long n, long long off, int nr, const Cx<T>* y, int mm,
                         Cx<T>* acc, const EngCtx& e) {
  using C = Cx<T>;
  for (int i0 = e.warp; i0 < mm; i0 += 4 * ENG_WARPS) {
    T sr[4] = {0, 0, 0, 0}, si[4] = {0, 0, 0, 0};
    for (int r = e.lane; r < nr; r += 32) {
      const C x = y[r];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int i = i0 + t * ENG_WARPS;
        if (i < mm) {
          const C a = V[(long long)i * n + off + r];
          sr[t] += a.x * x.x + a.y * x.y;
          si[t] += a.x * x.y - a.y * x.x;
        }
      }
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int i = i0 + t * ENG_WARPS;
      const T a = warp_sum(sr[t]), b = warp_sum(si[t]);
      if (e.lane == 0 && i < mm) acc[i] = mk2<T>(acc[i].x + a, acc[i].y + b);
    }
  }
}

// out[i] = sum_{g<G} pp[i G + g] for i < mm, the same order in every CTA;
// the partial loads of a lane are unrolled so that they are in flight together
template <class T>
__device__ void reduce_parts(const Cx<T>* pp, int G, int mm, Cx<T>* out, const EngCtx& e) {
  using C = Cx<T>;
  for (int i0 = e.warp; i0 < mm; i0 += 4 * ENG_WARPS) {
    T sr[4] = {0, 0, 0, 0}, si[4] = {0, 0, 0, 0};
#pragma unroll 10
    for (int g = e.lane; g < G; g += 32) {
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int i = i0 + t * ENG_WARPS;
        if (i < mm) {
          const C q = pp[(size_t)i * G + g];
          sr[t] += q.x;
          si[t] += q.y;
        }
      }
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int i = i0 + t * ENG_WARPS;
      const T a = warp_sum(sr[t]), b = warp_sum(si[t]);
      if (e.lane == 0 && i < mm) out[i] = mk2<T>(a, b);
    }
  }
}

// sum_{g<G} p[g], the same order in every CTA; ends with __syncthreads
template <class T>
__device__ T reduce_scalar(const T* p, int G, T* sh, const EngCtx& e) {
  if (e.warp == 0) {
    T a = (T)0;
#pragma unroll 10
    for (int g = e.lane; g < G; g += 32) a += p[g];
    a = warp_sum(a);
    if (e.lane == 0) sh[0] = a;
  }
  __syncthreads();
  const T r = sh[0];
  __syncthreads();
  return r;
}

// sum over the CTA of |y[r]|^2, r < nr, added to *acc by warp 0 / lane 0
template <class T>
__device__ void norm_acc(const Cx<T>* y, int nr, T* acc, const EngCtx& e) {
  if (e.warp == 0) {
    T s = (T)0;
    for (int r = e.lane; r < nr; r += 32) s += y[r].x * y[r].x + y[r].y * y[r].y;
    s = warp_sum(s);
    if (e.lane == 0) *acc += s;
  }
}

// ----------------------------------------------------- x-direction phases
// Schur x-convolution: CTA per z-point s; the four fields are handled by four
// groups of blockDim/4 threads, each with its own length-L shared-memory row.
// G = sum_j F_j e^{+i th} + sgn sum_{j>=1} F_j e^{-i th} (modes at +j and,
// times sgn, at L - j; one FFT), P = E G, H_i = (1/L) sum_l P e^{-i th_i}
// (one FFT, first Nk modes).  sgn = -1 for the first three fields, +1 for the
// fourth (the flipped cross term).
template <class T>
__device__ void ph_schur_x(const EngineOps& op, unsigned char* smraw, const EngCtx& e) {
  using C = typename CT2<T>::type;
  const int Nk = op.Nk, Mz = op.Mz, L = op.L;
  const int logL = ilog2_pow2(L);
  C* W = reinterpret_cast<C*>(smraw);           // L/2 twiddles
  const C* tw = (const C*)op.twS;
  const T* E = (const T*)op.E;
  const C* Fv = (const C*)op.Fv;
  C* Hv = (C*)op.Hv;
  for (int t = e.tid; t < (L >> 1); t += blockDim.x) W[t] = tw[t];
  const T invL = (T)1 / (T)L;
  if (schur_x_by_warp(L, (int)sizeof(C))) {
    // warp w: field w % 4 of the z-points b + (w / 4) G, b + (w / 4 + 2) G, ...
    __syncthreads();
    const int grp = e.warp & 3, nzs = ENG_WARPS / 4;
    C* P = W + (L >> 1) + e.warp * L;            // this warp's row
    const T sgn = (grp == 3) ? (T)1 : (T)-1;
    for (int s = e.b + (e.warp >> 2) * e.G; s < Mz; s += nzs * e.G) {
      for (int i = e.lane; i < L; i += 32) { P[i].x = (T)0; P[i].y = (T)0; }
      __syncwarp();
      for (int j = e.lane; j < Nk; j += 32) {
        const C f = Fv[((long long)grp * Nk + j) * Mz + s];
        P[j] = f;
        if (j > 0) { P[L - j].x = sgn * f.x; P[L - j].y = sgn * f.y; }
      }
      __syncwarp();
      warp_fft(P, L, logL, W, +1, e.lane);
      for (int l = e.lane; l < L; l += 32) {
        const T ev = E[(long long)l * Mz + s];
        P[l].x *= ev;
        P[l].y *= ev;
      }
      __syncwarp();
      warp_fft(P, L, logL, W, -1, e.lane);
      for (int i = e.lane; i < Nk; i += 32) {
        C o;
        o.x = P[i].x * invL;
        o.y = P[i].y * invL;
        Hv[((long long)grp * Nk + i) * Mz + s] = o;
      }
      __syncwarp();                              // the row is reused for the next z-point
    }
    return;
  }
  const int gsz = blockDim.x / 4, grp = e.tid / gsz, gt = e.tid % gsz;
  C* P = W + (L >> 1) + grp * L;                 // this group's row
  const T sgn = (grp == 3) ? (T)1 : (T)-1;
  for (int s = e.b; s < Mz; s += e.G) {
    __syncthreads();
    for (int i = gt; i < L; i += gsz) { P[i].x = (T)0; P[i].y = (T)0; }
    __syncthreads();
    for (int j = gt; j < Nk; j += gsz) {
      const C f = Fv[((long long)grp * Nk + j) * Mz + s];
      P[j] = f;
      if (j > 0) { P[L - j].x = sgn * f.x; P[L - j].y = sgn * f.y; }
    }
    __syncthreads();
    cta_fft(P, L, logL, W, +1, gt, gsz);
    for (int l = gt; l < L; l += gsz) {
      const T ev = E[(long long)l * Mz + s];
      P[l].x *= ev;
      P[l].y *= ev;
    }
    __syncthreads();
    cta_fft(P, L, logL, W, -1, gt, gsz);
    for (int i = gt; i < Nk; i += gsz) {
      C o;
      o.x = P[i].x * invL;
      o.y = P[i].y * invL;
      Hv[((long long)grp * Nk + i) * Mz + s] = o;
    }
  }
}

// theta x-phase: CTA per z-column j
template <class T>
__device__ void ph_theta_x(const EngineOps& op, unsigned char* smraw, const EngCtx& e) {
  using C = typename CT2<T>::type;
  const int Nk = op.Nk, N = op.N, Np = op.Np;
  C* xa = reinterpret_cast<C*>(smraw);
  C* xb = xa + Nk;
  C* W = xb + Nk;
  T* P = reinterpret_cast<T*>(W + Np);
  const C* X = (const C*)op.X;
  const C* tw = (const C*)op.twT;
  const T* ux = (const T*)op.ux;
  const T* uz = (const T*)op.uz;
  C* A = (C*)op.A;
  for (int i = e.tid; i < Np; i += blockDim.x) W[i] = tw[i];
  for (int j = e.b; j < N; j += e.G) {
    __syncthreads();
    for (int k = e.tid; k < Nk; k += blockDim.x) {
      xa[k] = X[(long long)k * N + j];
      xb[k] = X[(long long)(Nk + k) * N + j];
    }
    __syncthreads();
    for (int i = e.tid; i < Np; i += blockDim.x) {
      T a = xa[0].x, bv = xb[0].x;
      int idx = 0;
      for (int k = 1; k < Nk; ++k) {
        idx += i;
        if (idx >= Np) idx -= Np;
        const C t = W[idx];
        const T wk = (2 * k == Np) ? (T)1 : (T)2;
        a += wk * (xa[k].x * t.x - xa[k].y * t.y);
        bv += wk * (xb[k].x * t.x - xb[k].y * t.y);
      }
      const long long ee = (long long)i * N + j;
      P[i] = -(ux[ee] * a + uz[ee] * bv);
    }
    __syncthreads();
    const T inv = (T)1 / (T)Np;
    for (int base = 0; base < Nk; base += blockDim.x / 4) {
      const int k = base + e.tid / 4, part = e.tid & 3;
      T sr = 0, si = 0;
      if (k < Nk) {
        int idx = (int)(((long long)k * part) % Np);
        const int step = (int)(((long long)k * 4) % Np);
        for (int i = part; i < Np; i += 4) {
          const C t = W[idx];
          sr += P[i] * t.x;
          si -= P[i] * t.y;
          idx += step;
          if (idx >= Np) idx -= Np;
        }
      }
      sr += __shfl_xor_sync(0xffffffffu, sr, 1);
      si += __shfl_xor_sync(0xffffffffu, si, 1);
      sr += __shfl_xor_sync(0xffffffffu, sr, 2);
      si += __shfl_xor_sync(0xffffffffu, si, 2);
      if (k < Nk && part == 0) {
        C o;
        o.x = sr * inv;
        o.y = si * inv;
        A[(long long)k * N + j] = o;
      }
    }
  }
}


// ------------------------------------------------- block preconditioner
// double-float helpers: (s, c) is an unevaluated sum s + c of floats
__device__ __forceinline__ void df_add(float& s, float& c, float p) {
  const float t = s + p;
  const float bp = t - s;
  c += (s - (t - bp)) + (p - bp);
  s = t;
}
// (s, c) += (gh + gl) x for an FP32 x: exact product of the high part (FMA
// error term), the low part's product into the compensation
__device__ __forceinline__ void df_mac(float& s, float& c, float gh, float gl, float x) {
  const float p = gh * x;
  const float pe = fmaf(gh, x, -p);
  df_add(s, c, p);
  c += fmaf(gl, x, pe);
}

// z = palpha G_k v for the row task into S.z and (sub-0 CTA) Z_jv.
// T = double: FP64 GEMV.  T = float: the row v is exact in FP32 and G comes
// as (hi, lo) float pairs; the products G v cancel strongly for some rows, so
// they are summed in double-float arithmetic (lanes over output rows, warps
// over columns, warp partials merged with compensated adds in a fixed order)
// and rounded to FP32 once at the end.
template <class T>
__device__ void precond_row(const EngineOps& op, const EngineIO& io, int k, int sub, int jv,
                            long long off, EngSmem<T>& S, const EngCtx& e);

template <>
__device__ void precond_row<double>(const EngineOps& op, const EngineIO& io, int k, int sub, int jv,
                                    long long off, EngSmem<double>& S, const EngCtx& e) {
  const int N = op.N;
  double2* Z = io.Z;
  GemvArgs<double, 1> g;
  g.a[0] = (const double*)op.GpT + (long long)k * N * N;
  g.x[0] = S.v;
  for (int r0 = 0; r0 < N; r0 += RCH) {
    const int nr = min(RCH, N - r0);
    tgemv_chunk<double, 1>(g, N, r0, nr, N, S, e);
    for (int r = e.tid; r < nr; r += blockDim.x) {
      const double2 zz = make_double2(op.palpha * S.out[r].x, op.palpha * S.out[r].y);
      S.z[r0 + r] = zz;
      if (sub == 0) Z[(long long)jv * io.n + off + r0 + r] = zz;
    }
  }
}

template <>
__device__ void precond_row<float>(const EngineOps& op, const EngineIO& io, int k, int sub, int jv,
                                   long long off, EngSmem<float>& S, const EngCtx& e) {
  const int N = op.N;
  const float2* G = (const float2*)op.GpT + (long long)k * N * N;
  double2* Z = io.Z;
  float4* red = reinterpret_cast<float4*>(S.red);     // [warp][RCH] (re s, re c, im s, im c)
  const float pa = (float)op.palpha;
  for (int r0 = 0; r0 < N; r0 += RCH) {
    const int nr = min(RCH, N - r0);
    for (int rc = 0; rc < nr; rc += 32) {
      const int r = rc + e.lane;
      float sr = 0.f, cr = 0.f, si = 0.f, ci = 0.f;
      if (r < nr) {
#pragma unroll 4
        for (int c = e.warp; c < N; c += ENG_WARPS) {
          const float2 gg = G[(long long)c * N + r0 + r];
          const float2 x = S.v[c];
          df_mac(sr, cr, gg.x, gg.y, x.x);
          df_mac(si, ci, gg.x, gg.y, x.y);
        }
      }
      red[e.warp * RCH + r] = make_float4(sr, cr, si, ci);
    }
    __syncthreads();
    for (int r = e.tid; r < nr; r += blockDim.x) {
      float sr = 0.f, cr = 0.f, si = 0.f, ci = 0.f;
      for (int w = 0; w < ENG_WARPS; ++w) {
        const float4 q = red[w * RCH + r];
        df_add(sr, cr, q.x);
        cr += q.y;
        df_add(si, ci, q.z);
        ci += q.w;
      }
      S.z[r0 + r] = make_float2(pa * (sr + cr), pa * (si + ci));
      if (sub == 0)   // the full double-float value (the tau rows and x use it)
        Z[(long long)jv * io.n + off + r0 + r] =
            make_double2(op.palpha * ((double)sr + (double)cr), op.palpha * ((double)si + (double)ci));
    }
    __syncthreads();
  }
}

// The Schur z-contraction of the FP32 engine: out[m][r] = sum_c At[m][c ld +
// r0 + r] x[c] for m < 4 as tgemv_chunk, with matrices 0 and 1 (Zf, Z1 of
// this k) as (hi, lo) float pairs summed in double-float arithmetic and
// matrices 2, 3 in FP32.  Partials: per warp and row, (re s, re c, im s, im c)
// for m = 0, 1 and (re, im) for m = 2, 3, merged over the warps in a fixed
// order.  Ends with __syncthreads.
__device__ void tgemv4_df2(const float2* __restrict__ a0, const float2* __restrict__ a1,
                           const float* __restrict__ a2, const float* __restrict__ a3, long long ld,
                           int r0, int nr, int ncol, const float2* x, EngSmem<float>& S,
                           const EngCtx& e) {
  float4* red0 = reinterpret_cast<float4*>(S.red);               // [warp][RCH]
  float4* red1 = red0 + ENG_WARPS * RCH;
  float2* red2 = reinterpret_cast<float2*>(red1 + ENG_WARPS * RCH);
  float2* red3 = red2 + ENG_WARPS * RCH;
  for (int rc = 0; rc < nr; rc += 32) {
    const int r = rc + e.lane;
    float s0r = 0.f, c0r = 0.f, s0i = 0.f, c0i = 0.f, s1r = 0.f, c1r = 0.f, s1i = 0.f, c1i = 0.f;
    float p2r = 0.f, p2i = 0.f, p3r = 0.f, p3i = 0.f;
    if (r < nr) {
#pragma unroll 2
      for (int c = e.warp; c < ncol; c += ENG_WARPS) {
        const long long o = (long long)c * ld + r0 + r;
        const float2 xv = x[c];
        const float2 g0 = a0[o], g1 = a1[o];
        const float f2 = a2[o], f3 = a3[o];
        df_mac(s0r, c0r, g0.x, g0.y, xv.x);
        df_mac(s0i, c0i, g0.x, g0.y, xv.y);
        df_mac(s1r, c1r, g1.x, g1.y, xv.x);
        df_mac(s1i, c1i, g1.x, g1.y, xv.y);
        p2r += f2 * xv.x;
        p2i += f2 * xv.y;
        p3r += f3 * xv.x;
        p3i += f3 * xv.y;
      }
    }
    const int i = e.warp * RCH + r;
    red0[i] = make_float4(s0r, c0r, s0i, c0i);
    red1[i] = make_float4(s1r, c1r, s1i, c1i);
    red2[i] = make_float2(p2r, p2i);
    red3[i] = make_float2(p3r, p3i);
  }
  __syncthreads();
  for (int idx = e.tid; idx < 4 * nr; idx += blockDim.x) {
    const int m = idx / nr, r = idx - m * nr;
    float2 o;
    if (m < 2) {
      const float4* rd = m == 0 ? red0 : red1;
      float sr = 0.f, cr = 0.f, si = 0.f, ci = 0.f;
      for (int w = 0; w < ENG_WARPS; ++w) {
        const float4 q = rd[w * RCH + r];
        df_add(sr, cr, q.x);
        cr += q.y;
        df_add(si, ci, q.z);
        ci += q.w;
      }
      o = make_float2(sr + cr, si + ci);
    } else {
      const float2* rd = m == 2 ? red2 : red3;
      float sr = 0.f, si = 0.f;
      for (int w = 0; w < ENG_WARPS; ++w) {
        const float2 q = rd[w * RCH + r];
        sr += q.x;
        si += q.y;
      }
      o = make_float2(sr, si);
    }
    S.out[m * RCH + r] = o;
  }
  __syncthreads();
}

// The Schur epilogue GEMVs of the FP32 engine: out[0][r] = D2Zi (h0 + h1) in
// double-float arithmetic (D2Zi as (hi, lo) pairs, h0 and h1 multiplied
// separately, so their sum is not rounded first), out[1][r] = Zi xb and
// out[2][r] = DZi xc in FP32.  Ends with __syncthreads.
__device__ void tgemv3_epi_df(const float2* __restrict__ a0, const float* __restrict__ a1,
                              const float* __restrict__ a2, long long ld, int r0, int nr, int ncol,
                              const float2* h0, const float2* h1, const float2* xb,
                              const float2* xc, EngSmem<float>& S, const EngCtx& e) {
  float4* red0 = reinterpret_cast<float4*>(S.red);
  float4* red12 = red0 + ENG_WARPS * RCH;                         // (b re, b im, c re, c im)
  for (int rc = 0; rc < nr; rc += 32) {
    const int r = rc + e.lane;
    float sr = 0.f, cr = 0.f, si = 0.f, ci = 0.f, br = 0.f, bi = 0.f, qr = 0.f, qi = 0.f;
    if (r < nr) {
#pragma unroll 2
      for (int c = e.warp; c < ncol; c += ENG_WARPS) {
        const long long o = (long long)c * ld + r0 + r;
        const float2 g = a0[o];
        const float f1 = a1[o], f2 = a2[o];
        const float2 u = h0[c], v = h1[c], xb_ = xb[c], xc_ = xc[c];
        df_mac(sr, cr, g.x, g.y, u.x);
        df_mac(sr, cr, g.x, g.y, v.x);
        df_mac(si, ci, g.x, g.y, u.y);
        df_mac(si, ci, g.x, g.y, v.y);
        br += f1 * xb_.x;
        bi += f1 * xb_.y;
        qr += f2 * xc_.x;
        qi += f2 * xc_.y;
      }
    }
    const int i = e.warp * RCH + r;
    red0[i] = make_float4(sr, cr, si, ci);
    red12[i] = make_float4(br, bi, qr, qi);
  }
  __syncthreads();
  for (int r = e.tid; r < nr; r += blockDim.x) {
    float sr = 0.f, cr = 0.f, si = 0.f, ci = 0.f, br = 0.f, bi = 0.f, qr = 0.f, qi = 0.f;
    for (int w = 0; w < ENG_WARPS; ++w) {
      const float4 q = red0[w * RCH + r];
      df_add(sr, cr, q.x);
      cr += q.y;
      df_add(si, ci, q.z);
      ci += q.w;
      const float4 t = red12[w * RCH + r];
      br += t.x;
      bi += t.y;
      qr += t.z;
      qi += t.w;
    }
    S.out[r] = make_float2(sr + cr, si + ci);
    S.out[RCH + r] = make_float2(br, bi);
    S.out[2 * RCH + r] = make_float2(qr, qi);
  }
  __syncthreads();
}

// ------------------------------------------------------------ row phases
// prep: for each row task (k, sub): the row v_k of a new basis vector
//   mode 0: v = r * scale                 (start of a cycle; writes V_jv, Z_jv)
//   mode 1: v = (w - V coef) * scale      (Arnoldi step; writes V_jv, Z_jv)
//   mode 2: v = x                         (true residual: no preconditioner)
// then z = palpha G_k v (modes 0/1) and this sub's slice of the z-contraction.
template <class T>
__device__ void phase_prep(const EngineOps& op, const EngineIO& io, int mode, int jv, T scale,
                           const Cx<T>* coef, int mm, EngSmem<T>& S, const EngCtx& e,
                           PhaseClock* pc = nullptr, double scale64 = 1.0) {
  using C = Cx<T>;
  const int Nk = op.Nk, N = op.N;
  const long long n = io.n;
  const T* kxT = (const T*)op.kxT;
  C* V = reinterpret_cast<C*>(io.V);
  const C* Wv = reinterpret_cast<const C*>(io.w);
  const C* Rv = reinterpret_cast<const C*>(io.r);
  for (int t = e.b; t < e.ntask; t += e.G) {
    const int k = t / e.R, sub = t - (t / e.R) * e.R;
    const long long off = (long long)k * N;
    if (mode == 1) {
      combine_rows<T>(Wv, V, n, off, N, coef, mm, scale, S.v, nullptr, S, e);
      if (pc) pc->mark(EP_COMBINE);
    } else if (mode == 0) {
      for (int q = e.tid; q < N; q += blockDim.x) S.v[q] = x_scale<T>(Rv[off + q], scale);
      __syncthreads();
    } else {
      for (int q = e.tid; q < N; q += blockDim.x) {
        const double2 a = io.x[off + q];
        S.v[q] = mk2<T>((T)(a.x * scale64), (T)(a.y * scale64));
      }
      __syncthreads();
    }
    if (mode != 2) {
      if (sub == 0)
        for (int q = e.tid; q < N; q += blockDim.x) V[(long long)jv * n + off + q] = S.v[q];
      precond_row<T>(op, io, k, sub, jv, off, S, e);
      if (pc) pc->mark(EP_PRECOND);
    } else {
      for (int q = e.tid; q < N; q += blockDim.x) S.z[q] = S.v[q];
    }
    __syncthreads();
    const T kk = kxT[k];
    if (op.kind == 0) {
      // Fv[b][k][s] = c_b(k) sum_q Z_b(k)[s][q] z[q], c = (1, 2 k^2, 1, k)
      const int Mz = op.Mz;
      const int rc = (Mz + e.R - 1) / e.R;
      const int s_lo = sub * rc, s_hi = min(Mz, s_lo + rc);
      const long long MN = (long long)Mz * N;
      GemvArgs<T, 4> g;
      g.a[0] = (const T*)op.ZfT;
      g.a[1] = (const T*)op.Z1T + (long long)k * MN;
      g.a[2] = (const T*)op.Z2T + (long long)k * MN;
      g.a[3] = (const T*)op.Z3T + (long long)k * MN;
      g.x[0] = g.x[1] = g.x[2] = g.x[3] = S.z;
      C* Fv = (C*)op.Fv;
      const long long KM = (long long)Nk * Mz;
      const T c1 = (T)2 * kk * kk;
      for (int s0 = s_lo; s0 < s_hi; s0 += RCH) {
        const int nr = min(RCH, s_hi - s0);
        if constexpr (std::is_same<T, float>::value)
          tgemv4_df2((const float2*)op.ZfT2, (const float2*)op.Z1T2 + (long long)k * MN, g.a[2], g.a[3],
                     Mz, s0, nr, N, S.z, S, e);
        else
          tgemv_chunk<T, 4>(g, Mz, s0, nr, N, S, e);
        for (int r = e.tid; r < nr; r += blockDim.x) {
          const long long base = (long long)k * Mz + s0 + r;
          const C f0 = S.out[r], f1 = S.out[RCH + r], f2 = S.out[2 * RCH + r], f3 = S.out[3 * RCH + r];
          Fv[base] = f0;
          Fv[KM + base] = x_scale<T>(f1, c1);
          Fv[2 * KM + base] = f2;
          Fv[3 * KM + base] = x_scale<T>(f3, kk);
        }
      }
    } else {
      // X0[k][j] = i k (V z)[j], X1[k][j] = (VD z)[j]
      const int rc = (N + e.R - 1) / e.R;
      const int j_lo = sub * rc, j_hi = min(N, j_lo + rc);
      GemvArgs<T, 2> g;
      g.a[0] = (const T*)op.tVT;
      g.a[1] = (const T*)op.tVDT;
      g.x[0] = g.x[1] = S.z;
      C* X = (C*)op.X;
      for (int j0 = j_lo; j0 < j_hi; j0 += RCH) {
        const int nr = min(RCH, j_hi - j0);
        tgemv_chunk<T, 2>(g, N, j0, nr, N, S, e);
        for (int r = e.tid; r < nr; r += blockDim.x) {
          const C a = S.out[r], d = S.out[RCH + r];
          X[off + j0 + r] = mk2<T>(-kk * a.y, kk * a.x);
          X[(long long)(Nk + k) * N + j0 + r] = d;
        }
      }
    }
    __syncthreads();
    if (pc) pc->mark(EP_CONTRACT);
  }
}

// post: epilogue rows [p_lo, p_hi) of each row task; the operator's input
// vector is zin.  Arnoldi mode writes w and adds V_i^H w (i < mm) to acc;
// residual mode (zin = x, FP64) writes r = b - A x and adds ||r||^2 to *nacc.
template <class T>
__device__ void phase_post(const EngineOps& op, const EngineIO& io, bool resid, const double2* zin,
                           double zscale, int mm, EngSmem<T>& S, Cx<T>* acc, T* nacc,
                           const EngCtx& e) {
  using C = Cx<T>;
  const int Nk = op.Nk, N = op.N;
  const long long n = io.n;
  const T* kxT = (const T*)op.kxT;
  const C* V = reinterpret_cast<const C*>(io.V);
  for (int t = e.b; t < e.ntask; t += e.G) {
    const int k = t / e.R, sub = t - (t / e.R) * e.R;
    const long long off = (long long)k * N;
    const int pc = (N + e.R - 1) / e.R;
    const int p_lo = sub * pc, p_hi = min(N, p_lo + pc);
    if (p_lo >= p_hi) continue;                 // uniform within the CTA
    const int pe = min(p_hi, N - 2);            // rows above the tau rows
    const T kk = kxT[k];
    // operator input row in T (the temperature epilogue needs it)
    for (int q = e.tid; q < N; q += blockDim.x) {
      const double2 a = zin[off + q];
      S.v[q] = mk2<T>((T)(a.x * zscale), (T)(a.y * zscale));
    }
    if (op.kind == 0) {
      const int Mz = op.Mz;
      const C* Hv = (const C*)op.Hv;
      const long long KM = (long long)Nk * Mz;
      const T k2 = kk * kk;
      for (int q = e.tid; q < Mz; q += blockDim.x) {
        const long long i0 = (long long)k * Mz + q;
        const C h0 = Hv[i0], h1 = Hv[KM + i0], h2 = Hv[2 * KM + i0], h3 = Hv[3 * KM + i0];
        if constexpr (std::is_same<T, float>::value) {
          S.aux[q] = h0;                 // h0 and h1 kept apart: D2Zi (h0 + h1) is summed in double-float
          S.aux[3 * Mz + q] = h1;
        } else {
          S.aux[q] = x_add<T>(h0, h1);
        }
        S.aux[Mz + q] = mk2<T>((T)2 * k2 * h2.x - k2 * h0.x, (T)2 * k2 * h2.y - k2 * h0.y);
        S.aux[2 * Mz + q] = h3;
      }
      __syncthreads();
      if constexpr (std::is_same<T, float>::value) {
        for (int p0 = p_lo; p0 < pe; p0 += RCH) {
          const int nr = min(RCH, pe - p0);
          tgemv3_epi_df((const float2*)op.D2ZiT2, (const float*)op.ZiT, (const float*)op.DZiT, N, p0, nr,
                        Mz, S.aux, S.aux + 3 * Mz, S.aux + Mz, S.aux + 2 * Mz, S, e);
          for (int r = e.tid; r < nr; r += blockDim.x) {
            const C a = S.out[r], b = S.out[RCH + r], c = S.out[2 * RCH + r];
            S.w[p0 - p_lo + r] = mk2<T>(a.x + b.x - (T)4 * kk * c.x, a.y + b.y - (T)4 * kk * c.y);
          }
        }
      } else {
      GemvArgs<T, 3> g;
      g.a[0] = (const T*)op.D2ZiT;
      g.a[1] = (const T*)op.ZiT;
      g.a[2] = (const T*)op.DZiT;
      g.x[0] = S.aux;
      g.x[1] = S.aux + Mz;
      g.x[2] = S.aux + 2 * Mz;
      for (int p0 = p_lo; p0 < pe; p0 += RCH) {
        const int nr = min(RCH, pe - p0);
        tgemv_chunk<T, 3>(g, N, p0, nr, Mz, S, e);
        for (int r = e.tid; r < nr; r += blockDim.x) {
          const C a = S.out[r], b = S.out[RCH + r], c = S.out[2 * RCH + r];
          S.w[p0 - p_lo + r] = mk2<T>(a.x + b.x - (T)4 * kk * c.x, a.y + b.y - (T)4 * kk * c.y);
        }
      }
      }
    } else {
      const C* A = (const C*)op.A;
      for (int q = e.tid; q < N; q += blockDim.x) S.aux[q] = A[off + q];
      __syncthreads();
      GemvArgs<T, 2> g;
      g.a[0] = (const T*)op.tD2T;
      g.a[1] = (const T*)op.tViT;
      g.x[0] = S.v;
      g.x[1] = S.aux;
      const T k2 = kk * kk, a0 = (T)op.a0;
      for (int p0 = p_lo; p0 < pe; p0 += RCH) {
        const int nr = min(RCH, pe - p0);
        tgemv_chunk<T, 2>(g, N, p0, nr, N, S, e);
        for (int r = e.tid; r < nr; r += blockDim.x) {
          const C l = S.out[r], a = S.out[RCH + r];
          const C vn = S.v[p0 + r];
          // a0 v - (D2 v - k^2 v) - Vi A
          S.w[p0 - p_lo + r] = mk2<T>((a0 * vn.x - (l.x - k2 * vn.x)) - a.x,
                                      (a0 * vn.y - (l.y - k2 * vn.y)) - a.y);
        }
      }
    }
    // tau rows N-2, N-1: the boundary values of the input, in FP64 from the
    // FP64 input (these sums cancel strongly; one warp each)
    for (int p = max(p_lo, N - 2) + e.warp; p < p_hi; p += ENG_WARPS) {
      const double* Vr = op.V64 + (p == N - 2 ? 0 : (long long)(N - 1) * N);
      double sr = 0.0, si = 0.0;
      for (int m = e.lane; m < N; m += 32) {
        const double2 a = zin[off + m];
        sr += a.x * Vr[m];
        si += a.y * Vr[m];
      }
      sr = warp_sum(sr) * zscale;
      si = warp_sum(si) * zscale;
      if (e.lane == 0) S.w[p - p_lo] = mk2<T>((T)sr, (T)si);
    }
    __syncthreads();
    const int np = p_hi - p_lo;
    if (!resid) {
      C* W = reinterpret_cast<C*>(io.w);
      for (int r = e.tid; r < np; r += blockDim.x) W[off + p_lo + r] = S.w[r];
      dots_acc<T>(V, n, off + p_lo, np, S.w, mm, acc, e);
    } else {
      C* Rv = reinterpret_cast<C*>(io.r);
      for (int r = e.tid; r < np; r += blockDim.x) {
        const double2 bb = io.b[off + p_lo + r];
        const C rr = mk2<T>((T)(bb.x * zscale - (double)S.w[r].x), (T)(bb.y * zscale - (double)S.w[r].y));
        Rv[off + p_lo + r] = rr;
        S.w[r] = rr;
      }
      __syncthreads();
      norm_acc<T>(S.w, np, nacc, e);
    }
    __syncthreads();
  }
}

// update: w' = w - V coef on the owned rows (in place in io.w); then the dots
// V_i^H w' (i < mm_dots) into acc and ||w'||^2 into *nacc
template <class T>
__device__ void phase_update(const EngineOps& op, const EngineIO& io, const Cx<T>* coef, int mm,
                             int mm_dots, EngSmem<T>& S, Cx<T>* acc, T* nacc, const EngCtx& e) {
  using C = Cx<T>;
  const int N = op.N;
  const long long n = io.n;
  C* W = reinterpret_cast<C*>(io.w);
  const C* V = reinterpret_cast<const C*>(io.V);
  for (int t = e.b; t < e.ntask; t += e.G) {
    const int k = t / e.R, sub = t - (t / e.R) * e.R;
    const long long off = (long long)k * N;
    const int pc = (N + e.R - 1) / e.R;
    const int p_lo = sub * pc, p_hi = min(N, p_lo + pc);
    if (p_lo >= p_hi) continue;
    const int np = p_hi - p_lo;
    combine_rows<T>(W, V, n, off + p_lo, np, coef, mm, (T)1, S.w, W, S, e);
    if (mm_dots > 0) dots_acc<T>(V, n, off + p_lo, np, S.w, mm_dots, acc, e);
    norm_acc<T>(S.w, np, nacc, e);
    __syncthreads();
  }
}

// ------------------------------------------------------------- the engine
// Per-CTA shared state of one solve (every CTA holds identical values).
template <class T>
struct EngShared {
  T sh[8];
  Cx<T> h1[ENG_MAXM], h2[ENG_MAXM], hc[ENG_MAXM + 1], acc[ENG_MAXM];
  T cs[ENG_MAXM];
  Cx<T> sn[ENG_MAXM], g[ENG_MAXM + 1], y[ENG_MAXM];
  T nacc, hh;
  int flag;
  double part[ENG_WARPS];
  double b64;
};

// The CTAs of one solve: the whole grid (single-solve launches) or the
// group [cta0, cta0 + G) of a batched launch, CTA b of G.
__device__ __forceinline__ EngCtx eng_ctx_group(const EngineOps& op, int G, int b) {
  EngCtx e;
  e.G = G; e.b = b; e.tid = threadIdx.x; e.lane = e.tid & 31; e.warp = e.tid >> 5;
  e.gw = e.b * ENG_WARPS + e.warp;
  e.nw = e.G * ENG_WARPS;
  e.R = op.Nk <= e.G ? e.G / op.Nk : 1;
  e.ntask = op.Nk * e.R;
  return e;
}
__device__ __forceinline__ EngCtx eng_ctx(const EngineOps& op) {
  return eng_ctx_group(op, gridDim.x, blockIdx.x);
}

// Barrier over the CTAs of one solve.  GridBar: the cooperative grid barrier
// of a single-solve launch.  GroupBar: the CTAs of one solve inside a batched
// launch (every CTA of the launch is co-resident: cooperative launch) meet on
// an arrival counter and a generation word of their own in global memory, so
// the solves of a batch never wait for one another.  Thread 0 of each CTA
// arrives (release), the last arrival resets the counter and advances the
// generation (release), the others wait for the generation to move
// (acquire).  The wait is bounded: after timeout_ns of %globaltimer the CTA
// raises the group's *err (and the launch's *any) and stops waiting, and
// every later barrier of that group returns at once, so a group whose
// barrier could not complete still ends (all loops of a solve are bounded),
// its result is marked failed and the host reports the error; the other
// groups of the launch are not affected.
struct GridBar {
  cg::grid_group g;
  __device__ void sync() { g.sync(); }
};

struct GroupBar {
  unsigned int* cnt;
  unsigned int* gen;
  int G;
  int* err;
  int* any;
  long long timeout_ns;
  __device__ void sync() {
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned int my;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(my) : "l"(gen) : "memory");
      __threadfence();
      unsigned int arrived;
      asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;"
                   : "=r"(arrived) : "l"(cnt) : "memory");
      if (arrived == (unsigned int)G - 1) {
        asm volatile("st.relaxed.gpu.global.u32 [%0], 0;" ::"l"(cnt) : "memory");
        asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(gen), "r"(my + 1u) : "memory");
      } else {
        const long long t0 = global_ns();
        unsigned int now = my;
        int spins = 0;
        while (true) {
          asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(now) : "l"(gen) : "memory");
          if (now != my) break;
          if (*(volatile int*)err) break;
          if ((++spins & 63) == 0 && global_ns() - t0 > timeout_ns) {
            atomicExch(err, 1);
            atomicExch(any, 1);
            break;
          }
          __nanosleep(32);
        }
      }
      __threadfence();
    }
    __syncthreads();
  }
};

// One right-preconditioned FGMRES solve of A x = io.b (x -> io.x, FP64) to
// the relative tolerance io.rtol within io.maxiter Arnoldi steps; every CTA
// of the cooperative grid calls it.  -> info (0 converged, 1 not, 2
// breakdown, 3 non-finite data) and the Arnoldi steps taken.
template <class T, class Bar>
__device__ void fgmres_solve(const EngineOps& op, const EngineIO& io, EngShared<T>& Q,
                             unsigned char* smraw, const EngCtx& e, Bar& grid,
                             PhaseClock& pc, int& info_out, int& total_out) {
  using C = Cx<T>;
  T* sh = Q.sh;
  C *s_h1 = Q.h1, *s_h2 = Q.h2, *s_hc = Q.hc, *s_acc = Q.acc;
  T* s_cs = Q.cs;
  C *s_sn = Q.sn, *s_g = Q.g, *s_y = Q.y;
  T& s_nacc = Q.nacc;
  T& s_hh = Q.hh;
  int& s_flag = Q.flag;
  EngSmem<T> S = eng_carve<T>(smraw, op.N, op.Mz);
  const long long n = io.n;
  const int m = io.restart;
  const long long per = (n + e.G - 1) / e.G;
  const long long lo = (long long)e.b * per, hi = min(n, lo + per);
  C* pp1 = reinterpret_cast<C*>(io.part);
  C* pp2 = pp1 + (size_t)(m + 1) * e.G;
  T* np1 = reinterpret_cast<T*>(io.npart);       // ||.||^2 partials
  T* np2 = np1 + e.G;                            // second set (exact norm)
  double2* Zv = io.Z;
  C* Rv = reinterpret_cast<C*>(io.r);
  C* Hm = reinterpret_cast<C*>(io.H);
  C* Yv = reinterpret_cast<C*>(io.y);
  // heavy cancellation in ||w'||^2 - ||h2||^2 below this fraction of ||w'||^2
  // means the Pythagorean norm has lost too many digits
  const T cancel = std::is_same<T, float>::value ? (T)1e-2 : (T)1e-4;

  // x = 0; b64 = ||b|| in FP64; the Krylov process works on r = b / b64 (unit
  // norm, so nothing in T under- or overflows whatever the problem's scale)
  // and x is accumulated in units of b64
  double b64;
  {
    double s = 0.0;
    for (long long t = lo + e.tid; t < hi; t += blockDim.x) {
      io.x[t] = make_double2(0.0, 0.0);
      const double2 bb = io.b[t];
      s += bb.x * bb.x + bb.y * bb.y;
    }
    s = warp_sum(s);
    if (e.lane == 0) Q.part[e.warp] = s;
    __syncthreads();
    double* npd = io.npart;
    if (e.tid == 0) {
      double a = 0.0;
      for (int q = 0; q < ENG_WARPS; ++q) a += Q.part[q];
      npd[e.b] = a;
    }
    grid.sync();
    if (e.warp == 0) {
      double a = 0.0;
#pragma unroll 10
      for (int g = e.lane; g < e.G; g += 32) a += npd[g];
      a = warp_sum(a);
      if (e.lane == 0) Q.b64 = sqrt(a);
    }
    __syncthreads();
    b64 = Q.b64;
  }
  const double inv64 = (b64 > 0.0 && isfinite(b64)) ? 1.0 / b64 : 0.0;
  for (long long t = lo + e.tid; t < hi; t += blockDim.x) {
    const double2 bb = io.b[t];
    Rv[t] = mk2<T>((T)(bb.x * inv64), (T)(bb.y * inv64));
  }
  grid.sync();                                  // prep reads whole rows of r
  T beta = (T)1;
  const T tol = (T)io.rtol;
  int total = 0, info = 1;
  if (b64 == 0.0) info = 0;
  if (!isfinite(b64)) info = 3;               // non-finite right-hand side
  while (info == 1 && total < io.maxiter) {
    // V0 = r / beta, Z0 = M V0 and its z-contraction
    phase_prep<T>(op, io, 0, 0, (T)1 / beta, nullptr, 0, S, e);
    for (int i = e.tid; i <= m; i += blockDim.x) s_g[i] = mk2<T>((T)0, (T)0);
    __syncthreads();
    if (e.tid == 0) s_g[0] = mk2<T>(beta, (T)0);
    grid.sync();
    pc.mark(EP_START);
    int kc = 0;
    for (int j = 0; j < m; ++j) {
      // x-direction convolution of A z_j
      if (op.kind == 0) ph_schur_x<T>(op, smraw, e);
      else ph_theta_x<T>(op, smraw, e);
      __syncthreads();
      pc.mark(EP_XCONV);
      grid.sync();
      pc.mark(EP_XCONV_WAIT);
      // epilogue w = A z_j + first-pass dots
      const int mm = j + 1;
      for (int i = e.tid; i < mm; i += blockDim.x) s_acc[i] = mk2<T>((T)0, (T)0);
      __syncthreads();
      phase_post<T>(op, io, false, Zv + (long long)j * n, 1.0, mm, S, s_acc, nullptr, e);
      __syncthreads();
      for (int i = e.tid; i < mm; i += blockDim.x) pp1[(size_t)i * e.G + e.b] = s_acc[i];
      __syncthreads();
      pc.mark(EP_POST);
      grid.sync();
      pc.mark(EP_POST_WAIT);
      // h1 = V^H w; w' = w - V h1; second-pass dots and ||w'||^2
      reduce_parts<T>(pp1, e.G, mm, s_h1, e);
      for (int i = e.tid; i < mm; i += blockDim.x) s_acc[i] = mk2<T>((T)0, (T)0);
      if (e.tid == 0) s_nacc = (T)0;
      __syncthreads();
      pc.mark(EP_UPD_RED);
      phase_update<T>(op, io, s_h1, mm, mm, S, s_acc, &s_nacc, e);
      __syncthreads();
      for (int i = e.tid; i < mm; i += blockDim.x) pp2[(size_t)i * e.G + e.b] = s_acc[i];
      if (e.tid == 0) np1[e.b] = s_nacc;
      __syncthreads();
      pc.mark(EP_UPDATE);
      grid.sync();
      pc.mark(EP_UPDATE_WAIT);
      // h2 = V^H w', ||w''||^2 = ||w'||^2 - ||h2||^2
      reduce_parts<T>(pp2, e.G, mm, s_h2, e);
      const T wn2 = reduce_scalar<T>(np1, e.G, sh, e);     // ends with __syncthreads
      if (e.warp == 0) {
        T a = (T)0;
        for (int i = e.lane; i < mm; i += 32) a += s_h2[i].x * s_h2[i].x + s_h2[i].y * s_h2[i].y;
        a = warp_sum(a);
        if (e.lane == 0) s_hh = a;
      }
      __syncthreads();
      const T hh = s_hh;
      pc.mark(EP_NEXT_RED);
      if (!isfinite(wn2) || !isfinite(hh)) {     // non-finite operator output: give up
        info = 3;
        break;
      }
      T hn2 = wn2 - hh;
      bool subtracted = false;
      if (!(hn2 > cancel * wn2)) {
        // heavy cancellation: form w'' = w' - V h2 and take its exact norm
        if (e.tid == 0) s_nacc = (T)0;
        __syncthreads();
        phase_update<T>(op, io, s_h2, mm, 0, S, nullptr, &s_nacc, e);
        __syncthreads();
        // second partial array: other CTAs may still be reading np1 here
        if (e.tid == 0) np2[e.b] = s_nacc;
        grid.sync();
        hn2 = reduce_scalar<T>(np2, e.G, sh, e);
        subtracted = true;
        pc.mark(EP_EXACT);
      }
      const T hn = sqrt(hn2 > (T)0 ? hn2 : (T)0);
      // Givens update of column j (every CTA, identical data)
      if (e.tid == 0) {
        for (int i = 0; i < mm; ++i) s_hc[i] = x_add<T>(s_h1[i], s_h2[i]);
        s_hc[j + 1] = mk2<T>(hn, (T)0);
        for (int i = 0; i < j; ++i) {
          const T c = s_cs[i];
          const C sv = s_sn[i];
          const C hi0 = s_hc[i], hi1 = s_hc[i + 1];
          s_hc[i] = x_add<T>(x_scale<T>(hi0, c), x_mul<T>(sv, hi1));
          s_hc[i + 1] = x_add<T>(x_mul<T>(mk2<T>(-sv.x, sv.y), hi0), x_scale<T>(hi1, c));  // -conj(s) h_i + c h_{i+1}
        }
        const C a = s_hc[j], bb = s_hc[j + 1];
        const T aa = x_abs<T>(a), bba = x_abs<T>(bb);
        T c;
        C sv, rjj;
        if (bba == (T)0) { c = (T)1; sv = mk2<T>((T)0, (T)0); rjj = a; }
        else if (aa == (T)0) { c = (T)0; sv = mk2<T>(bb.x / bba, -bb.y / bba); rjj = mk2<T>(bba, (T)0); }
        else {
          const T den = sqrt(aa * aa + bba * bba);
          c = aa / den;
          sv = x_scale<T>(x_div<T>(x_conj<T>(bb), x_conj<T>(a)), c);
          rjj = x_scale<T>(x_div<T>(mk2<T>((T)1, (T)0), x_conj<T>(a)), c * (aa * aa + bba * bba));
        }
        s_cs[j] = c;
        s_sn[j] = sv;
        s_hc[j] = rjj;
        const C gj = s_g[j], gj1 = s_g[j + 1];
        s_g[j] = x_add<T>(x_scale<T>(gj, c), x_mul<T>(sv, gj1));
        s_g[j + 1] = x_add<T>(x_mul<T>(mk2<T>(-sv.x, sv.y), gj), x_scale<T>(gj1, c));
        const T rn = x_abs<T>(s_g[j + 1]);
        s_flag = (rn <= tol) ? 1 : ((hn == (T)0) ? 2 : 0);
      }
      __syncthreads();
      pc.mark(EP_GIVENS);
      if (e.b == 0) {
        C* Hc = Hm + (size_t)j * (m + 1);     // rotated column j, rows 0..j
        for (int i = e.tid; i <= j; i += blockDim.x) Hc[i] = s_hc[i];
      }
      const int fl = s_flag;
      ++total;
      kc = j + 1;
      const bool stop = fl != 0 || j + 1 == m || total >= io.maxiter;
      if (!stop)
        phase_prep<T>(op, io, 1, j + 1, (T)1 / hn, s_h2, subtracted ? 0 : mm, S, e, &pc);
      grid.sync();
      pc.mark(EP_NEXT_WAIT);
      if (stop) {
        if (fl == 1) info = 0;
        else if (fl == 2) info = 2;
        break;
      }
    }
    if (kc == 0) break;
    // y = H[:k,:k]^{-1} g[:k]: column sweep by CTA 0 (the column of H is
    // contiguous in the column-major layout), then x += Z y everywhere (FP64)
    if (e.b == 0) {
      for (int i = e.tid; i < kc; i += blockDim.x) s_y[i] = s_g[i];
      __syncthreads();
      for (int q = kc - 1; q >= 0; --q) {
        const C* Hq = Hm + (size_t)q * (m + 1);
        if (e.tid == 0) s_y[q] = x_div<T>(s_y[q], Hq[q]);
        __syncthreads();
        const C yq = s_y[q];
        for (int i = e.tid; i < q; i += blockDim.x) s_y[i] = x_sub<T>(s_y[i], x_mul<T>(Hq[i], yq));
        __syncthreads();
      }
      for (int i = e.tid; i < kc; i += blockDim.x) Yv[i] = s_y[i];
    }
    grid.sync();
    for (long long t = lo + e.tid; t < hi; t += blockDim.x) {
      double ar = 0.0, ai = 0.0;
      for (int q = 0; q < kc; ++q) {
        const C yq = Yv[q];
        const double2 z = Zv[(long long)q * n + t];
        ar += (double)yq.x * z.x - (double)yq.y * z.y;
        ai += (double)yq.x * z.y + (double)yq.y * z.x;
      }
      io.x[t].x += b64 * ar;
      io.x[t].y += b64 * ai;
    }
    grid.sync();
    pc.mark(EP_LSQ);
    if (info != 1 || total >= io.maxiter) break;
    // true residual at the restart: r = b - A x
    phase_prep<T>(op, io, 2, 0, (T)1, nullptr, 0, S, e, nullptr, inv64);
    grid.sync();
    if (op.kind == 0) ph_schur_x<T>(op, smraw, e);
    else ph_theta_x<T>(op, smraw, e);
    grid.sync();
    if (e.tid == 0) s_nacc = (T)0;
    __syncthreads();
    phase_post<T>(op, io, true, io.x, inv64, 0, S, nullptr, &s_nacc, e);
    __syncthreads();
    if (e.tid == 0) np1[e.b] = s_nacc;
    grid.sync();
    beta = sqrt(reduce_scalar<T>(np1, e.G, sh, e));
    pc.mark(EP_RESID);
    if (beta <= tol) { info = 0; break; }
    if (!isfinite(beta)) { info = 3; break; }
  }
  info_out = info;
  total_out = total;
}

template <class T>
__global__ void __launch_bounds__(ENG_THREADS, 2) smc_fgmres_engine_kernel(EngineOps op, EngineIO io) {
  GridBar grid{cg::this_grid()};
  extern __shared__ __align__(256) unsigned char smraw[];
  __shared__ EngShared<T> Q;
  const EngCtx e = eng_ctx(op);
  PhaseClock pc;
  pc.init(io.phase_cycles, e);
  int info = 1, total = 0;
  fgmres_solve<T, GridBar>(op, io, Q, smraw, e, grid, pc, info, total);
  if (e.b == 0 && e.tid == 0) {
    io.result[0] = info;
    io.result[1] = total;
  }
  pc.finish();
}

// Iterative refinement of one solve: FP64 outer residuals r = b - A64 x
// (the FP64 operator phases), FP32 inner FGMRES solves of A32 e = r to
// max(0.3 tol / ||r||, floor), x += e, until ||r|| <= rtol ||b||, at most 12
// outer passes and maxiter inner Arnoldi steps in all.  -> info, inner
// steps, outer passes, final relative residual (in the caller's registers).
struct RefineShared {
  EngShared<float> Q;
  double red[8];
  double part[ENG_WARPS];
  double nacc64;
};

template <class Bar>
__device__ void refine_solve(const EngineOps& op32, const EngineOps& op64, const EngineIO& io,
                             const RefineIO& rf, RefineShared& RS, unsigned char* smraw,
                             const EngCtx& e, Bar& grid, PhaseClock& pc, int& info_out,
                             int& total_out, int& outer_out, double& rel_out) {
  EngShared<float>& Q = RS.Q;
  double* s_red = RS.red;
  double* s_part = RS.part;
  double& s_nacc64 = RS.nacc64;
  const long long n = io.n;
  const long long per = (n + e.G - 1) / e.G;
  const long long lo = (long long)e.b * per, hi = min(n, lo + per);
  double* npr = io.npart + e.G;           // the inner solve uses io.npart[0, G)
  // x = 0 (or the guess the caller left in x), r = b, ||b||
  {
    double s = 0.0;
    for (long long t = lo + e.tid; t < hi; t += blockDim.x) {
      const double2 bb = rf.b[t];
      if (!rf.warm) rf.x[t] = make_double2(0.0, 0.0);
      rf.r[t] = bb;
      s += bb.x * bb.x + bb.y * bb.y;
    }
    s = warp_sum(s);
    if (e.lane == 0) s_part[e.warp] = s;
    __syncthreads();
    if (e.tid == 0) {
      double a = 0.0;
      for (int q = 0; q < ENG_WARPS; ++q) a += s_part[q];
      npr[e.b] = a;
    }
    grid.sync();
  }
  const double bn = sqrt(reduce_scalar<double>(npr, e.G, s_red, e));
  const double tol = rf.rtol * bn;
  double beta = bn;
  int total = 0, outer = 0, info = 1;
  EngSmem<double> S64 = eng_carve<double>(smraw, op64.N, op64.Mz);
  EngineIO o64 = io;
  o64.b = rf.b;
  o64.x = rf.x;
  o64.r = rf.r;
  // r = b - A64 x and its norm: the FP64 pass that ends every outer iteration
  auto residual64 = [&]() -> double {
    phase_prep<double>(op64, o64, 2, 0, 1.0, nullptr, 0, S64, e, nullptr, 1.0);
    grid.sync();
    pc.mark(EP_REF_PREP);
    if (op64.kind == 0) ph_schur_x<double>(op64, smraw, e);
    else ph_theta_x<double>(op64, smraw, e);
    grid.sync();
    pc.mark(EP_REF_XCONV);
    if (e.tid == 0) s_nacc64 = 0.0;
    __syncthreads();
    phase_post<double>(op64, o64, true, rf.x, 1.0, 0, S64, nullptr, &s_nacc64, e);
    __syncthreads();
    if (e.tid == 0) npr[e.b] = s_nacc64;
    grid.sync();
    return sqrt(reduce_scalar<double>(npr, e.G, s_red, e));
  };
  if (rf.warm && bn > 0.0 && isfinite(bn)) {
    // start from the caller's guess (the previous solve's solution): its
    // residual instead of b; a non-finite one falls back to x = 0
    beta = residual64();
    if (!isfinite(beta)) {
      for (long long t = lo + e.tid; t < hi; t += blockDim.x) {
        rf.x[t] = make_double2(0.0, 0.0);
        rf.r[t] = rf.b[t];
      }
      grid.sync();
      beta = bn;
    }
  }
  while (outer < 12) {
    if (beta <= tol) { info = 0; break; }
    if (!isfinite(beta)) { info = 3; break; }
    if (total >= rf.maxiter) break;
    EngineIO in = io;
    in.b = rf.r;
    in.x = rf.e;
    in.rtol = fmax(0.3 * tol / beta, rf.floor);
    in.maxiter = rf.maxiter - total;
    int inf = 1, its = 0;
    fgmres_solve<float, Bar>(op32, in, Q, smraw, e, grid, pc, inf, its);
    total += its;
    if (inf == 3) { info = 3; break; }
    for (long long t = lo + e.tid; t < hi; t += blockDim.x) {
      const double2 a = rf.x[t], d = rf.e[t];
      rf.x[t] = make_double2(a.x + d.x, a.y + d.y);
    }
    grid.sync();
    pc.mark(EP_REF_XUPD);
    beta = residual64();                            // r = b - A64 x
    pc.mark(EP_REF_POST);
    ++outer;
    pc.mark(EP_REFINE);
    if (its == 0 && beta > tol) break;             // no progress possible
  }
  if (beta <= tol && info != 3) info = 0;
  info_out = info;
  total_out = total;
  outer_out = outer;
  rel_out = beta / fmax(bn, 1e-300);
}

// The whole refinement of one solve in one cooperative launch.
__global__ void __launch_bounds__(ENG_THREADS, 2) smc_refine_engine_kernel(EngineOps op32, EngineOps op64,
                                                                           EngineIO io, RefineIO rf) {
  GridBar grid{cg::this_grid()};
  extern __shared__ __align__(256) unsigned char smraw[];
  __shared__ RefineShared RS;
  const EngCtx e = eng_ctx(op32);
  PhaseClock pc;
  pc.init(io.phase_cycles, e);
  int info = 1, total = 0, outer = 0;
  double rel = 0.0;
  refine_solve<GridBar>(op32, op64, io, rf, RS, smraw, e, grid, pc, info, total, outer, rel);
  if (e.b == 0 && e.tid == 0) {
    io.result[0] = info;
    io.result[1] = total;
    io.result[2] = outer;
    rf.res[0] = rel;
  }
  pc.finish();
}

// The refinement solves of independent systems (any mix of Schur and
// temperature operators and grid sizes) in one cooperative launch: slot j
// owns the CTAs [cta0, cta0 + G) and a group barrier of its own, and starts
// with its first solve.  When a solve has ended, CTA 0 of the group -- after a
// last group barrier, so no CTA of the group touches the solve's buffers any
// more -- writes the result block to host-mapped memory and then the done
// word, so the host thread that owns the solve goes on while the batch runs.
// With a feed, the group's leader then claims the next solve the host has
// published (waiting up to idle_ns for one, claiming none after life_ns),
// hands the ticket to its CTAs through the group barrier, and every CTA of
// the group copies that solve's descriptor into shared memory and runs it on
// the slot's CTAs: a slot whose solve converged in a few Arnoldi steps does
// not idle until the slowest solve of the launch ends.
__device__ __forceinline__ int ld_acquire_sys(const volatile int* p) {
  int v;
  asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__global__ void __launch_bounds__(ENG_THREADS, 2) smc_refine_batch_kernel(
    const __grid_constant__ RefineBatch B) {
  extern __shared__ __align__(256) unsigned char smraw[];
  __shared__ RefineShared RS;
  __shared__ __align__(16) RefineJob sJ;
  int j = 0;
  while (j + 1 < B.njobs && (int)blockIdx.x >= B.job[j + 1].cta0) ++j;
  const int cta0 = B.job[j].cta0, G = B.job[j].G;
  unsigned int* sb = B.slot_bar + 4 * j;
  GroupBar bar{sb, sb + 1, G, reinterpret_cast<int*>(sb + 2), B.err, B.timeout_ns};
  const long long t_start = global_ns();
  const RefineJob* J = &B.job[j];
  while (true) {
    const EngCtx e = eng_ctx_group(J->op32, G, (int)blockIdx.x - cta0);
    PhaseClock pc;
    pc.init(nullptr, e);
    int info = 1, total = 0, outer = 0;
    double rel = 0.0;
    refine_solve<GroupBar>(J->op32, J->op64, J->io, J->rf, RS, smraw, e, bar, pc, info, total,
                           outer, rel);
    bar.sync();
    if (e.b == 0 && e.tid == 0) {
      volatile EngineJobResult* out = J->out;
      out->info = info;
      out->iters = total;
      out->outer = outer;
      out->rel = rel;
      out->failed = *(volatile int*)(sb + 2);
      __threadfence_system();
      out->done = J->seq;
    }
    if (!B.feed) break;
    // the next solve: the leader claims a published ticket (bounded wait)
    if (e.b == 0 && e.tid == 0) {
      int t = -1;
      const long long t0 = global_ns();
      while (true) {
        const long long now = global_ns();
        if (now - t_start > B.life_ns || now - t0 > B.idle_ns) break;
        if (*(volatile int*)(sb + 2)) break;          // this group's barrier timed out
        const int pub = ld_acquire_sys(&B.feed->published);
        const int c = *(volatile int*)B.claimed;
        if (c < pub) {
          if (atomicCAS(B.claimed, c, c + 1) == c) { t = c; break; }
          continue;
        }
        __nanosleep(256);
      }
      *(volatile int*)(B.slot_ticket + j) = t;
    }
    bar.sync();
    const int t = *(volatile int*)(B.slot_ticket + j);
    if (t < 0) break;
    // every CTA copies the solve's descriptor (published before the ticket)
    const volatile unsigned int* src =
        reinterpret_cast<const volatile unsigned int*>(&B.feed->ring[t % BATCH_FEED_CAP]);
    unsigned int* dst = reinterpret_cast<unsigned int*>(&sJ);
    for (int w = threadIdx.x; w < (int)(sizeof(RefineJob) / 4); w += blockDim.x) dst[w] = src[w];
    __syncthreads();
    J = &sJ;
  }
}

template <class T>
static size_t engine_smem(const EngineOps& op) {
  using C = Cx<T>;
  const size_t a = (size_t)(op.L / 2 + (schur_x_by_warp(op.L, (int)sizeof(C)) ? 8 : 4) * op.L) *
                   sizeof(C);                                                         // Schur x
  const size_t b = (size_t)(2 * op.Nk + op.Np) * sizeof(C) + op.Np * sizeof(T);     // theta x
  const size_t rows = eng_rows_bytes<T>(op.N, op.kind == 0 ? op.Mz : 0);
  size_t s = rows;
  if (op.kind == 0 && a > s) s = a;
  if (op.kind == 1 && b > s) s = b;
  return s;
}

template <class T>
static void engine_launch(const Ctx& c, const EngineOps& op, const EngineIO& io) {
  const size_t sm = engine_smem<T>(op);
  auto kern = smc_fgmres_engine_kernel<T>;
  allow_max_smem((const void*)kern);
  int per_sm = 0;
  SMC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, ENG_THREADS, sm));
  if (per_sm < 1) {
    cudaFuncAttributes fa;
    cudaFuncGetAttributes(&fa, (const void*)kern);
    throw std::runtime_error("fgmres engine: kernel cannot be co-resident (kind " +
                             std::to_string(op.kind) + ", N " + std::to_string(op.N) + ", Mz " +
                             std::to_string(op.Mz) + ", L " + std::to_string(op.L) + ", Np " +
                             std::to_string(op.Np) + ", dynamic smem " + std::to_string(sm) +
                             ", static smem " + std::to_string(fa.sharedSizeBytes) + ", max dynamic " +
                             std::to_string(fa.maxDynamicSharedSizeBytes) + ", regs " +
                             std::to_string(fa.numRegs) + ")");
  }
  int G = c.num_sms * (per_sm >= 2 ? 2 : 1);
  if (io.grid_cap > 0 && io.grid_cap < G) G = io.grid_cap;
  if (G > io.max_grid) throw std::runtime_error("fgmres engine: partial buffers too small");
  EngineOps o = op;
  EngineIO i = io;
  void* args[] = {(void*)&o, (void*)&i};
  CoopGuard guard(c.s);
  SMC_CUDA(cudaLaunchCooperativeKernel((void*)kern, dim3(G), dim3(ENG_THREADS), args, sm, c.s));
  SMC_LAUNCH_CHECK(c);
}

void fgmres_refine_engine(const Ctx& c, const EngineOps& op32, const EngineOps& op64,
                          const EngineIO& io, const RefineIO& rf) {
  if (io.restart + 1 > ENG_MAXM) throw std::runtime_error("fgmres engine: restart above 99");
  const size_t s32 = engine_smem<float>(op32), s64 = engine_smem<double>(op64);
  const size_t sm = s32 > s64 ? s32 : s64;
  auto kern = smc_refine_engine_kernel;
  allow_max_smem((const void*)kern);
  int per_sm = 0;
  SMC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, ENG_THREADS, sm));
  if (per_sm < 1) throw std::runtime_error("refinement engine: kernel cannot be co-resident");
  int G = c.num_sms * (per_sm >= 2 ? 2 : 1);
  if (io.grid_cap > 0 && io.grid_cap < G) G = io.grid_cap;
  if (G > io.max_grid) throw std::runtime_error("refinement engine: partial buffers too small");
  EngineOps a = op32, b = op64;
  EngineIO i = io;
  RefineIO r = rf;
  void* args[] = {(void*)&a, (void*)&b, (void*)&i, (void*)&r};
  CoopGuard guard(c.s);
  SMC_CUDA(cudaLaunchCooperativeKernel((void*)kern, dim3(G), dim3(ENG_THREADS), args, sm, c.s));
  SMC_LAUNCH_CHECK(c);
}

size_t refine_engine_smem(const EngineOps& op32, const EngineOps& op64) {
  const size_t s32 = engine_smem<float>(op32), s64 = engine_smem<double>(op64);
  return s32 > s64 ? s32 : s64;
}

int refine_batch_capacity(size_t smem, int num_sms) {
  auto kern = smc_refine_batch_kernel;
  allow_max_smem((const void*)kern);
  int per_sm = 0;
  SMC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, ENG_THREADS, smem));
  return per_sm * num_sms;
}

void refine_batch_launch(cudaStream_t s, const RefineBatch& B, size_t smem) {
  auto kern = smc_refine_batch_kernel;
  allow_max_smem((const void*)kern);
  if (!B.slot_bar) throw std::runtime_error("refine batch: no slot barrier words");
  int G = 0;
  for (int j = 0; j < B.njobs; ++j) {
    if (B.job[j].cta0 != G) throw std::runtime_error("refine batch: CTA ranges not contiguous");
    if (B.job[j].io.restart + 1 > ENG_MAXM) throw std::runtime_error("refine batch: restart above 99");
    if (B.job[j].G > B.job[j].io.max_grid) throw std::runtime_error("refine batch: partials too small");
    G += B.job[j].G;
  }
  RefineBatch b = B;
  void* args[] = {(void*)&b};
  SMC_CUDA(cudaLaunchCooperativeKernel((void*)kern, dim3(G), dim3(ENG_THREADS), args, smem, s));
  SMC_CUDA(cudaGetLastError());
}

void fgmres_engine(const Ctx& c, const EngineOps& op, const EngineIO& io, bool fp32) {
  if (io.restart + 1 > ENG_MAXM) throw std::runtime_error("fgmres engine: restart above 99");
  if (fp32) engine_launch<float>(c, op, io);
  else engine_launch<double>(c, op, io);
}

// ------------------------------------------------------------- transpose
template <class To>
__global__ void smc_transpose_kernel(const double* __restrict__ in, To* __restrict__ out,
                                     long long rows, long long cols) {
  __shared__ double tile[32][33];
  const long long bofs = (long long)blockIdx.z * rows * cols;
  const long long c0 = (long long)blockIdx.x * 32, r0 = (long long)blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const long long r = r0 + i, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[i][threadIdx.x] = in[bofs + r * cols + c];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const long long c = c0 + i, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[bofs + c * rows + r] = (To)tile[threadIdx.x][i];
  }
}

template <class To>
static void transpose_impl(const Ctx& c, const double* in, To* out, long long rows, long long cols,
                           int batch) {
  dim3 grid(ceil_div(cols, 32), ceil_div(rows, 32), batch);
  smc_transpose_kernel<To><<<grid, dim3(32, 8), 0, c.s>>>(in, out, rows, cols);
  SMC_LAUNCH_CHECK(c);
}
void transpose_as(const Ctx& c, const double* in, float* out, long long rows, long long cols, int batch) {
  transpose_impl<float>(c, in, out, rows, cols, batch);
}
void transpose_as(const Ctx& c, const double* in, double* out, long long rows, long long cols, int batch) {
  transpose_impl<double>(c, in, out, rows, cols, batch);
}

__global__ void smc_transpose_split_kernel(const double* __restrict__ in, float2* __restrict__ out,
                                           long long rows, long long cols) {
  __shared__ double tile[32][33];
  const long long bofs = (long long)blockIdx.z * rows * cols;
  const long long c0 = (long long)blockIdx.x * 32, r0 = (long long)blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const long long r = r0 + i, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[i][threadIdx.x] = in[bofs + r * cols + c];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const long long c = c0 + i, r = r0 + threadIdx.x;
    if (r < rows && c < cols) {
      const double v = tile[threadIdx.x][i];
      const float hi = (float)v;
      out[bofs + c * rows + r] = make_float2(hi, (float)(v - (double)hi));
    }
  }
}

void transpose_split(const Ctx& c, const double* in, float2* out, long long rows, long long cols,
                     int batch) {
  dim3 grid(ceil_div(cols, 32), ceil_div(rows, 32), batch);
  smc_transpose_split_kernel<<<grid, dim3(32, 8), 0, c.s>>>(in, out, rows, cols);
  SMC_LAUNCH_CHECK(c);
}

}  // namespace smc
