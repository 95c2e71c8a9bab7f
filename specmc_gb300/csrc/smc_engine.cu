// Persistent Krylov engine of the fast form: one cooperative launch runs a
// whole right-preconditioned FGMRES solve (core/krylov_fgmres.py:60-179) on
// the device -- preconditioner, operator, Arnoldi (CGS2) and the Givens
// least-squares update -- with grid barriers between dependent phases and no
// host round trip per iteration.
//
// Operators: the fused Schur matvec (stokes/lagged_stokes.py:202-220) or the
// fused temperature matvec (implicit_theta.py:354-383), in working precision
// T (float: the inner solves of the mixed form; double: FP64).  Krylov
// vectors, the Hessenberg matrix and the Givens data stay FP64.
//
// Uniform control: every branch that decides how many grid barriers a CTA
// executes depends only on data every CTA reads after the same barrier
// (values reduced in the same order by every CTA, or a flag written by CTA 0
// before a barrier), and every loop is bounded by the restart length and the
// iteration budget, so all CTAs execute the same sequence of barriers.
#include <cooperative_groups.h>

#include <type_traits>

#include "smc_internal.cuh"
#include "smc_engine.cuh"

namespace cg = cooperative_groups;

namespace smc {

template <class T> struct CT2;
template <> struct CT2<double> { using type = double2; };
template <> struct CT2<float> { using type = float2; };

struct EngCtx {
  int G, b, tid, lane, warp, gw, nw;   // grid size, block, thread, lane, warp, global warp, #warps
};

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------- phases
// out[k][n] = alpha sum_m Gp[k][n][m] in[k][m]       (warp per output)
__device__ void ph_precond(const EngineOps& op, const double2* in, double2* out, const EngCtx& e) {
  const long long no = (long long)op.Nk * op.N;
  for (long long o = e.gw; o < no; o += e.nw) {
    const int k = (int)(o / op.N), n = (int)(o % op.N);
    const double* g = op.Gp + ((long long)k * op.N + n) * op.N;
    const double2* r = in + (long long)k * op.N;
    double sr = 0.0, si = 0.0;
    for (int m = e.lane; m < op.N; m += 32) {
      sr += g[m] * r[m].x;
      si += g[m] * r[m].y;
    }
    sr = warp_sum(sr);
    si = warp_sum(si);
    if (e.lane == 0) out[o] = make_double2(op.palpha * sr, op.palpha * si);
  }
}

template <class T>
__device__ void ph_convert(const EngineOps& op, const double2* in, typename CT2<T>::type* out,
                           long long n, const EngCtx& e) {
  for (long long t = (long long)e.b * blockDim.x + e.tid; t < n; t += (long long)e.G * blockDim.x) {
    typename CT2<T>::type v;
    v.x = (T)in[t].x;
    v.y = (T)in[t].y;
    out[t] = v;
  }
}

// Schur forward: Fv[b][k][s] = c_b(k) sum_q Z_b(k)[s][q] v[k][q]; one warp
// per (k, s) forms all four fields from one read of v_k (4 independent sums)
template <class T>
__device__ void ph_schur_fwd(const EngineOps& op, const typename CT2<T>::type* v, const EngCtx& e) {
  using C = typename CT2<T>::type;
  const long long total = (long long)op.Nk * op.Mz;
  const long long MN = (long long)op.Mz * op.N;
  C* Fv = (C*)op.Fv;
  for (long long o = e.gw; o < total; o += e.nw) {
    const int s = (int)(o % op.Mz);
    const int k = (int)(o / op.Mz);
    const T* z0 = (const T*)op.Zf + (long long)s * op.N;
    const T* z1 = (const T*)op.Z1 + (long long)k * MN + (long long)s * op.N;
    const T* z2 = (const T*)op.Z2 + (long long)k * MN + (long long)s * op.N;
    const T* z3 = (const T*)op.Z3 + (long long)k * MN + (long long)s * op.N;
    const C* vk = v + (long long)k * op.N;
    T a0 = 0, b0 = 0, a1 = 0, b1 = 0, a2 = 0, b2 = 0, a3 = 0, b3 = 0;
    for (int q = e.lane; q < op.N; q += 32) {
      const C x = vk[q];
      const T w0 = z0[q], w1 = z1[q], w2 = z2[q], w3 = z3[q];
      a0 += w0 * x.x; b0 += w0 * x.y;
      a1 += w1 * x.x; b1 += w1 * x.y;
      a2 += w2 * x.x; b2 += w2 * x.y;
      a3 += w3 * x.x; b3 += w3 * x.y;
    }
    for (int d = 16; d > 0; d >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, d); b0 += __shfl_xor_sync(0xffffffffu, b0, d);
      a1 += __shfl_xor_sync(0xffffffffu, a1, d); b1 += __shfl_xor_sync(0xffffffffu, b1, d);
      a2 += __shfl_xor_sync(0xffffffffu, a2, d); b2 += __shfl_xor_sync(0xffffffffu, b2, d);
      a3 += __shfl_xor_sync(0xffffffffu, a3, d); b3 += __shfl_xor_sync(0xffffffffu, b3, d);
    }
    if (e.lane == 0) {
      const T kk = ((const T*)op.kxT)[k];
      const T c1 = (T)2 * kk * kk;
      const long long KM = (long long)op.Nk * op.Mz;
      const long long base = (long long)k * op.Mz + s;
      C r;
      r.x = a0; r.y = b0; Fv[base] = r;
      r.x = c1 * a1; r.y = c1 * b1; Fv[KM + base] = r;
      r.x = a2; r.y = b2; Fv[2 * KM + base] = r;
      r.x = kk * a3; r.y = kk * b3; Fv[3 * KM + base] = r;
    }
  }
}

// Schur x-convolution: CTA per z-point s; the four fields are handled by
// four groups of blockDim/4 threads with their own shared-memory slices
template <class T>
__device__ void ph_schur_x(const EngineOps& op, unsigned char* smraw, const EngCtx& e) {
  using C = typename CT2<T>::type;
  const int Nk = op.Nk, Mz = op.Mz, L = op.L;
  const int gsz = blockDim.x / 4, grp = e.tid / gsz, gt = e.tid % gsz;
  C* W = reinterpret_cast<C*>(smraw);           // L twiddles
  C* F = W + L + grp * (Nk + L);                 // this group's field
  C* P = F + Nk;
  const C* tw = (const C*)op.twS;
  const T* E = (const T*)op.E;
  const C* Fv = (const C*)op.Fv;
  C* Hv = (C*)op.Hv;
  for (int t = e.tid; t < L; t += blockDim.x) W[t] = tw[t];
  const T sgn = (grp == 3) ? (T)1 : (T)-1;
  const T ap = (T)1 + sgn, am = (T)1 - sgn;
  const T invL = (T)1 / (T)L;
  for (int s = e.b; s < Mz; s += e.G) {
    __syncthreads();
    for (int j = gt; j < Nk; j += gsz) F[j] = Fv[((long long)grp * Nk + j) * Mz + s];
    __syncthreads();
    for (int l = gt; l < L; l += gsz) {
      T gr = F[0].x, gi = F[0].y;
      int idx = 0;
      for (int j = 1; j < Nk; ++j) {
        idx += l;
        if (idx >= L) idx -= L;
        const C t = W[idx];
        const C f = F[j];
        gr += ap * (f.x * t.x) - am * (f.y * t.y);
        gi += ap * (f.y * t.x) + am * (f.x * t.y);
      }
      const T ev = E[(long long)l * Mz + s];
      P[l].x = ev * gr;
      P[l].y = ev * gi;
    }
    __syncthreads();
    // 4 consecutive threads per output mode i (groups are warp-aligned)
    for (int base = 0; base < Nk; base += gsz / 4) {
      const int i = base + gt / 4, part = gt & 3;
      T hr = 0, hi = 0;
      if (i < Nk) {
        int idx = (int)(((long long)i * part) % L);
        const int step = (int)(((long long)i * 4) % L);
        for (int l = part; l < L; l += 4) {
          const C t = W[idx];
          const C p = P[l];
          hr += p.x * t.x + p.y * t.y;
          hi += p.y * t.x - p.x * t.y;
          idx += step;
          if (idx >= L) idx -= L;
        }
      }
      hr += __shfl_xor_sync(0xffffffffu, hr, 1);
      hi += __shfl_xor_sync(0xffffffffu, hi, 1);
      hr += __shfl_xor_sync(0xffffffffu, hr, 2);
      hi += __shfl_xor_sync(0xffffffffu, hi, 2);
      if (i < Nk && part == 0) {
        C o;
        o.x = hr * invL;
        o.y = hi * invL;
        Hv[((long long)grp * Nk + i) * Mz + s] = o;
      }
    }
  }
}

// Schur epilogue (warp per output (k, p)); tau rows from the FP64 input
template <class T>
__device__ void ph_schur_out(const EngineOps& op, const double2* v, double2* out, const EngCtx& e) {
  using C = typename CT2<T>::type;
  const int Nk = op.Nk, N = op.N, Mz = op.Mz;
  const C* Hv = (const C*)op.Hv;
  const long long KM = (long long)Nk * Mz;
  for (long long o = e.gw; o < (long long)Nk * N; o += e.nw) {
    const int k = (int)(o / N), p = (int)(o % N);
    if (p >= N - 2) {
      const double* Vr = op.V64 + (p == N - 2 ? 0 : (long long)(N - 1) * N);
      const double2* vk = v + (long long)k * N;
      double sr = 0, si = 0;
      for (int m = e.lane; m < N; m += 32) { sr += vk[m].x * Vr[m]; si += vk[m].y * Vr[m]; }
      sr = warp_sum(sr);
      si = warp_sum(si);
      if (e.lane == 0) out[o] = make_double2(sr, si);
      continue;
    }
    const C* H0 = Hv + (long long)k * Mz;
    const C* H1 = H0 + KM;
    const C* H2 = H1 + KM;
    const C* H3 = H2 + KM;
    const T* a = (const T*)op.D2Zi + (long long)p * Mz;
    const T* z = (const T*)op.Zi + (long long)p * Mz;
    const T* dd = (const T*)op.DZi + (long long)p * Mz;
    const T kk = ((const T*)op.kxT)[k];
    const T k2 = kk * kk;
    T ar = 0, ai = 0, br = 0, bi = 0, cr = 0, ci = 0;
    for (int q = e.lane; q < Mz; q += 32) {
      const T as = a[q], zs = z[q], ds = dd[q];
      const C h0 = H0[q], h1 = H1[q], h2 = H2[q], h3 = H3[q];
      ar += as * (h0.x + h1.x);
      ai += as * (h0.y + h1.y);
      br += zs * ((T)2 * k2 * h2.x - k2 * h0.x);
      bi += zs * ((T)2 * k2 * h2.y - k2 * h0.y);
      cr += ds * h3.x;
      ci += ds * h3.y;
    }
    ar = warp_sum(ar); ai = warp_sum(ai); br = warp_sum(br);
    bi = warp_sum(bi); cr = warp_sum(cr); ci = warp_sum(ci);
    if (e.lane == 0) {
      const T r = ar + br - (T)4 * kk * cr;
      const T im = ai + bi - (T)4 * kk * ci;
      out[o] = make_double2((double)r, (double)im);
    }
  }
}

// theta z-synthesis: X0[k][j] = i k (V v_k)[j], X1 = (VD v_k)[j]
template <class T>
__device__ void ph_theta_z(const EngineOps& op, const typename CT2<T>::type* v, const EngCtx& e) {
  using C = typename CT2<T>::type;
  const int Nk = op.Nk, N = op.N;
  C* X = (C*)op.X;
  for (long long o = e.gw; o < (long long)Nk * N; o += e.nw) {
    const int k = (int)(o / N), j = (int)(o % N);
    const T* a = (const T*)op.tV + (long long)j * N;
    const T* d = (const T*)op.tVD + (long long)j * N;
    const C* vk = v + (long long)k * N;
    T ar = 0, ai = 0, dr = 0, di = 0;
    for (int q = e.lane; q < N; q += 32) {
      const C x = vk[q];
      ar += a[q] * x.x;
      ai += a[q] * x.y;
      dr += d[q] * x.x;
      di += d[q] * x.y;
    }
    ar = warp_sum(ar); ai = warp_sum(ai); dr = warp_sum(dr); di = warp_sum(di);
    if (e.lane == 0) {
      const T kk = ((const T*)op.kxT)[k];
      C o0, o1;
      o0.x = -kk * ai;
      o0.y = kk * ar;
      o1.x = dr;
      o1.y = di;
      X[(long long)k * N + j] = o0;
      X[(long long)(Nk + k) * N + j] = o1;
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

// theta epilogue: out = a0 v - (D2 v - k^2 v) - Vi A ; tau rows (warp per output)
template <class T>
__device__ void ph_theta_out(const EngineOps& op, const double2* v, const typename CT2<T>::type* vT,
                             double2* out, const EngCtx& e) {
  using C = typename CT2<T>::type;
  const int Nk = op.Nk, N = op.N;
  const C* A = (const C*)op.A;
  for (long long o = e.gw; o < (long long)Nk * N; o += e.nw) {
    const int k = (int)(o / N), n = (int)(o % N);
    const double2* vk = v + (long long)k * N;
    if (n >= N - 2) {
      const double* Vr = op.V64 + (n == N - 2 ? 0 : (long long)(N - 1) * N);
      double sr = 0, si = 0;
      for (int m = e.lane; m < N; m += 32) { sr += vk[m].x * Vr[m]; si += vk[m].y * Vr[m]; }
      sr = warp_sum(sr);
      si = warp_sum(si);
      if (e.lane == 0) out[o] = make_double2(sr, si);
      continue;
    }
    const T* dr = (const T*)op.tD2 + (long long)n * N;
    const T* vi = (const T*)op.tVi + (long long)n * N;
    const C* Ak = A + (long long)k * N;
    const C* vTk = vT + (long long)k * N;
    T lr = 0, li = 0, ar = 0, ai = 0;
    for (int m = e.lane; m < N; m += 32) {
      lr += dr[m] * vTk[m].x;
      li += dr[m] * vTk[m].y;
      ar += vi[m] * Ak[m].x;
      ai += vi[m] * Ak[m].y;
    }
    lr = warp_sum(lr); li = warp_sum(li); ar = warp_sum(ar); ai = warp_sum(ai);
    if (e.lane == 0) {
      const double k2 = op.kx[k] * op.kx[k];
      const double2 vn = vk[n];
      const double Lr = (double)lr - k2 * vn.x, Li = (double)li - k2 * vn.y;
      out[o] = make_double2((op.a0 * vn.x - Lr) - (double)ar, (op.a0 * vn.y - Li) - (double)ai);
    }
  }
}

// out = A(in) (both FP64 vectors); grid barriers between the phases
template <class T>
__device__ void apply_op(const EngineOps& op, const double2* in, double2* out, unsigned char* sm,
                         const EngCtx& e, cg::grid_group& grid) {
  using C = typename CT2<T>::type;
  const long long n = (long long)op.Nk * op.N;
  const C* vT;
  if (std::is_same<T, float>::value) {
    ph_convert<T>(op, in, (C*)op.vT, n, e);
    grid.sync();
    vT = (const C*)op.vT;
  } else {
    vT = reinterpret_cast<const C*>(in);
  }
  if (op.kind == 0) {
    ph_schur_fwd<T>(op, vT, e);
    grid.sync();
    ph_schur_x<T>(op, sm, e);
    grid.sync();
    ph_schur_out<T>(op, in, out, e);
  } else {
    ph_theta_z<T>(op, vT, e);
    grid.sync();
    ph_theta_x<T>(op, sm, e);
    grid.sync();
    ph_theta_out<T>(op, in, vT, out, e);
  }
  grid.sync();
}

// sum of the G per-CTA partials (same order in every CTA)
__device__ double grid_total(const double* part, int G, const EngCtx& e, double* sh) {
  if (e.warp == 0) {
    double a = 0.0;
    for (int g = e.lane; g < G; g += 32) a += part[g];
    a = warp_sum(a);
    if (e.lane == 0) sh[0] = a;
  }
  __syncthreads();
  double r = sh[0];
  __syncthreads();
  return r;
}

// ||x|| over the grid (one barrier); every CTA returns the same value
__device__ double grid_norm(const double2* x, long long n, double* part, const EngCtx& e,
                            cg::grid_group& grid, double* sh) {
  const long long per = (n + e.G - 1) / e.G;
  const long long lo = (long long)e.b * per, hi = min(n, lo + per);
  double s = 0.0;
  for (long long t = lo + e.tid; t < hi; t += blockDim.x) s += x[t].x * x[t].x + x[t].y * x[t].y;
  s = warp_sum(s);
  if (e.lane == 0) sh[1 + e.warp] = s;
  __syncthreads();
  if (e.tid == 0) {
    double a = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) a += sh[1 + q];
    part[e.b] = a;
  }
  grid.sync();
  return sqrt(grid_total(part, e.G, e, sh));
}

// ------------------------------------------------------------- the engine
template <class T>
__global__ void __launch_bounds__(256) smc_fgmres_engine_kernel(EngineOps op, EngineIO io) {
  cg::grid_group grid = cg::this_grid();
  extern __shared__ unsigned char smraw[];
  __shared__ double sh[40];
  __shared__ double2 hcol[100], hsum[100];
  // Givens state, kept by CTA 0 in shared memory for the whole solve
  __shared__ double s_cs[100];
  __shared__ double2 s_sn[100], s_g[101], s_y[100];
  __shared__ int s_flag;
  EngCtx e;
  e.G = gridDim.x; e.b = blockIdx.x; e.tid = threadIdx.x; e.lane = e.tid & 31; e.warp = e.tid >> 5;
  e.gw = e.b * (blockDim.x >> 5) + e.warp;
  e.nw = e.G * (blockDim.x >> 5);
  const long long n = io.n;
  const int m = io.restart;
  const long long per = (n + e.G - 1) / e.G;
  const long long lo = (long long)e.b * per, hi = min(n, lo + per);

  // x = 0, r = b, beta = ||b||
  for (long long t = (long long)e.b * blockDim.x + e.tid; t < n; t += (long long)e.G * blockDim.x) {
    io.x[t] = make_double2(0.0, 0.0);
    io.r[t] = io.b[t];
  }
  double beta = grid_norm(io.b, n, io.npart, e, grid, sh);
  const double tol = io.rtol * beta;
  int total = 0, info = 1;
  if (beta <= tol) info = 0;
  while (info == 1 && total < io.maxiter) {
    // V0 = r / beta
    for (long long t = lo + e.tid; t < hi; t += blockDim.x) {
      double2 v = io.r[t];
      io.V[t] = make_double2(v.x / beta, v.y / beta);
    }
    if (e.b == 0) {
      for (int i = e.tid; i <= m; i += blockDim.x) s_g[i] = make_double2(0.0, 0.0);
      __syncthreads();
      if (e.tid == 0) s_g[0] = make_double2(beta, 0.0);
    }
    grid.sync();
    int k = 0;
    for (int j = 0; j < m; ++j) {
      if (total >= io.maxiter) { info = 1; break; }
      double2* Vj = io.V + (long long)j * n;
      double2* Zj = io.Z + (long long)j * n;
      ph_precond(op, Vj, Zj, e);
      grid.sync();
      apply_op<T>(op, Zj, io.w, smraw, e, grid);
      // ---- CGS2 of w against V_0..V_j (all CTAs end with identical hsum, hn)
      const int mm = j + 1;
      for (int i = e.tid; i < mm; i += blockDim.x) hsum[i] = make_double2(0.0, 0.0);
      __syncthreads();
      for (int pass = 0; pass < 2; ++pass) {
        double2* pp = io.part + (size_t)pass * e.G * (m + 1);
        for (int i = e.warp; i < mm; i += (blockDim.x >> 5)) {
          const double2* Vi = io.V + (long long)i * n;
          double sr = 0.0, si = 0.0;
          for (long long t = lo + e.lane; t < hi; t += 32) {
            const double2 a = Vi[t], x = io.w[t];
            sr += a.x * x.x + a.y * x.y;
            si += a.x * x.y - a.y * x.x;
          }
          sr = warp_sum(sr);
          si = warp_sum(si);
          if (e.lane == 0) pp[(size_t)e.b * (m + 1) + i] = make_double2(sr, si);
        }
        grid.sync();
        for (int i = e.warp; i < mm; i += (blockDim.x >> 5)) {
          double sr = 0.0, si = 0.0;
          for (int g = e.lane; g < e.G; g += 32) {
            const double2 q = pp[(size_t)g * (m + 1) + i];
            sr += q.x;
            si += q.y;
          }
          sr = warp_sum(sr);
          si = warp_sum(si);
          if (e.lane == 0) {
            hcol[i] = make_double2(sr, si);
            hsum[i] = cadd(hsum[i], hcol[i]);
          }
        }
        __syncthreads();
        for (long long t = lo + e.tid; t < hi; t += blockDim.x) {
          double2 x = io.w[t];
          for (int i = 0; i < mm; ++i) x = csub(x, cmul(hcol[i], io.V[(long long)i * n + t]));
          io.w[t] = x;
        }
        __syncthreads();
      }
      const double hn = grid_norm(io.w, n, io.npart, e, grid, sh);
      // ---- Givens update of column j (CTA 0, shared-memory state) and the
      //      stopping decision, published through global memory
      if (e.b == 0) {
        if (e.tid == 0) {
          hsum[j + 1] = make_double2(hn, 0.0);
          for (int i = 0; i < j; ++i) {
            const double c = s_cs[i];
            const double2 sv = s_sn[i];
            const double2 hi0 = hsum[i], hi1 = hsum[i + 1];
            const double2 t = cadd(cscale(hi0, c), cmul(sv, hi1));
            hsum[i + 1] = cadd(cmul(make_double2(-sv.x, sv.y), hi0), cscale(hi1, c));  // -conj(s) h_i + c h_{i+1}
            hsum[i] = t;
          }
          const double2 a = hsum[j], bb = hsum[j + 1];
          const double aa = hypot(a.x, a.y), bba = hypot(bb.x, bb.y);
          double c;
          double2 sv, rjj;
          if (bba == 0.0) { c = 1.0; sv = make_double2(0.0, 0.0); rjj = a; }
          else if (aa == 0.0) { c = 0.0; sv = make_double2(bb.x / bba, -bb.y / bba); rjj = make_double2(bba, 0.0); }
          else {
            const double den = sqrt(aa * aa + bba * bba);
            c = aa / den;
            sv = cscale(cdiv(cconj(bb), cconj(a)), c);
            rjj = cscale(cdiv(make_double2(1.0, 0.0), cconj(a)), c * (aa * aa + bba * bba));
          }
          s_cs[j] = c;
          s_sn[j] = sv;
          hsum[j] = rjj;
          hsum[j + 1] = make_double2(0.0, 0.0);
          const double2 gj = s_g[j], gj1 = s_g[j + 1];
          s_g[j] = cadd(cscale(gj, c), cmul(sv, gj1));
          s_g[j + 1] = cadd(cmul(make_double2(-sv.x, sv.y), gj), cscale(gj1, c));
          const double rn = hypot(s_g[j + 1].x, s_g[j + 1].y);
          s_flag = (rn <= tol) ? 1 : ((hn == 0.0) ? 2 : 0);
        }
        __syncthreads();
        double2* Hc = io.H + (size_t)j * (m + 1);     // rotated column j, rows 0..j
        for (int i = e.tid; i <= j; i += blockDim.x) Hc[i] = hsum[i];
        if (e.tid == 0) io.flag[0] = s_flag;
      }
      if (hn != 0.0) {
        double2* Vn = io.V + (long long)(j + 1) * n;
        for (long long t = lo + e.tid; t < hi; t += blockDim.x) {
          const double2 x = io.w[t];
          Vn[t] = make_double2(x.x / hn, x.y / hn);
        }
      }
      grid.sync();
      const int fl = *((volatile int*)io.flag);
      ++total;
      k = j + 1;
      if (fl == 1) { info = 0; break; }
      if (fl == 2) { info = 2; break; }
    }
    if (k == 0) break;
    // y = H[:k,:k]^{-1} g[:k]: column sweep by CTA 0 (the column of H is
    // contiguous in the column-major layout), then x += Z y everywhere
    if (e.b == 0) {
      for (int i = e.tid; i < k; i += blockDim.x) s_y[i] = s_g[i];
      __syncthreads();
      for (int q = k - 1; q >= 0; --q) {
        const double2* Hq = io.H + (size_t)q * (m + 1);
        if (e.tid == 0) s_y[q] = cdiv(s_y[q], Hq[q]);
        __syncthreads();
        const double2 yq = s_y[q];
        for (int i = e.tid; i < q; i += blockDim.x) s_y[i] = csub(s_y[i], cmul(Hq[i], yq));
        __syncthreads();
      }
      for (int i = e.tid; i < k; i += blockDim.x) io.y[i] = s_y[i];
    }
    grid.sync();
    for (long long t = lo + e.tid; t < hi; t += blockDim.x) {
      double2 acc = make_double2(0.0, 0.0);
      for (int q = 0; q < k; ++q) acc = cadd(acc, cmul(io.y[q], io.Z[(long long)q * n + t]));
      io.x[t] = cadd(io.x[t], acc);
    }
    grid.sync();
    if (info == 0 || info == 2) break;
    // true residual at the restart: r = b - A x
    apply_op<T>(op, io.x, io.r, smraw, e, grid);
    for (long long t = lo + e.tid; t < hi; t += blockDim.x) io.r[t] = csub(io.b[t], io.r[t]);
    grid.sync();
    beta = grid_norm(io.r, n, io.npart, e, grid, sh);
    if (beta <= tol) { info = 0; break; }
  }
  if (e.b == 0 && e.tid == 0) {
    io.result[0] = info;
    io.result[1] = total;
  }
}

template <class T>
static size_t engine_smem(const EngineOps& op) {
  using C = typename CT2<T>::type;
  size_t a = (size_t)(op.L + 4 * (op.Nk + op.L)) * sizeof(C);
  size_t b = (size_t)(2 * op.Nk + op.Np) * sizeof(C) + op.Np * sizeof(T);
  return a > b ? a : b;
}

template <class T>
static void engine_launch(const Ctx& c, const EngineOps& op, const EngineIO& io) {
  const size_t sm = engine_smem<T>(op);
  auto kern = smc_fgmres_engine_kernel<T>;
  if (sm > 48 * 1024)
    SMC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  int per_sm = 0;
  SMC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, sm));
  if (per_sm < 1) throw std::runtime_error("fgmres engine: kernel cannot be co-resident");
  const int G = c.num_sms * (per_sm >= 2 ? 2 : 1);
  if (G > io.max_grid) throw std::runtime_error("fgmres engine: partial buffers too small");
  EngineOps o = op;
  EngineIO i = io;
  void* args[] = {(void*)&o, (void*)&i};
  SMC_CUDA(cudaLaunchCooperativeKernel((void*)kern, dim3(G), dim3(256), args, sm, c.s));
  SMC_LAUNCH_CHECK(c);
}

void fgmres_engine(const Ctx& c, const EngineOps& op, const EngineIO& io, bool fp32) {
  if (io.restart + 1 > 100) throw std::runtime_error("fgmres engine: restart above 99");
  if (fp32) engine_launch<float>(c, op, io);
  else engine_launch<double>(c, op, io);
}

}  // namespace smc
