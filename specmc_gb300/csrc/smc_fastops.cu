// Fused operators of the fast (mixed) form.
//
//  * Schur matvec (stokes/lagged_stokes.py:202-220) in three launches: the
//    Green operator, D^2 and D are folded into per-wavenumber operators
//    Z1_k = Zf G_k, Z2_k = Zf D2 G_k, Z3_k = Zf D G_k (forward values at the
//    Mz CGL points of the pseudo-spectral product), and D^2, D into the
//    inverse (D2 Zi, D Zi), so the matvec is: 4 forward contractions ->
//    x-convolution with eta on the (L x Mz) grid -> one epilogue contraction.
//  * Temperature matvec (implicit_theta.py:354-383) in three launches:
//    z-synthesis of (ik v, D v) -> per z-column padded x-synthesis, advective
//    product, x-analysis -> V^{-1} contraction with the Helmholtz part.
//  * Cooperative CGS2 Arnoldi step over all SMs (FP64).
// Templated on the working real type T (double: FP64 operators; float: the
// inner-iteration operators of the mixed form).  Krylov vectors stay FP64 at
// the interface: inputs are read as double2 and converted, outputs written as
// double2.
#include <cooperative_groups.h>

#include <type_traits>

#include "smc_internal.cuh"
#include "smc_fastops.cuh"
#include "smc_fft.cuh"

namespace cg = cooperative_groups;

namespace smc {

template <class T> struct C2;
template <> struct C2<double> { using type = double2; };
template <> struct C2<float> { using type = float2; };

// ---------------------------------------------------------- Schur matvec
// Fv[b][k][s] = c_b(k) sum_q Z_b(k)[s][q] v[k][q]
//   b=0: Zf (shared), c=1 ; b=1: Z1_k, c=2k^2 ; b=2: Z2_k, c=1 ; b=3: Z3_k, c=k
// one warp per output (b, k, s); lanes split q (coalesced rows of Z)
template <class T>
__global__ void smc_fs_fwd_kernel(const typename C2<T>::type* __restrict__ v, const T* __restrict__ Zf,
                                  const T* __restrict__ Z1, const T* __restrict__ Z2,
                                  const T* __restrict__ Z3, const double* __restrict__ kx, int Nk,
                                  int N, int Mz, typename C2<T>::type* __restrict__ Fv) {
  const int lane = threadIdx.x & 31;
  const long long o = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const long long total = 4LL * Nk * Mz;
  if (o >= total) return;
  const int s = (int)(o % Mz);
  const int k = (int)((o / Mz) % Nk);
  const int b = (int)(o / ((long long)Mz * Nk));
  const long long MN = (long long)Mz * N;
  const T* Z = (b == 0) ? Zf : ((b == 1 ? Z1 : (b == 2 ? Z2 : Z3)) + (long long)k * MN);
  const T* zr = Z + (long long)s * N;
  const typename C2<T>::type* vk = v + (long long)k * N;
  T sr = 0, si = 0;
  for (int q = lane; q < N; q += 32) {
    const T w = zr[q];
    const typename C2<T>::type x = vk[q];
    sr += w * x.x;
    si += w * x.y;
  }
  for (int d = 16; d > 0; d >>= 1) {
    sr += __shfl_xor_sync(0xffffffffu, sr, d);
    si += __shfl_xor_sync(0xffffffffu, si, d);
  }
  if (lane == 0) {
    const double kk = kx[k];
    const T c = (T)(b == 1 ? 2.0 * kk * kk : (b == 3 ? kk : 1.0));
    typename C2<T>::type r;
    r.x = c * sr;
    r.y = c * si;
    Fv[((long long)b * Nk + k) * Mz + s] = r;
  }
}

// per (s, b): G(l) = sum_j F_j e^{+i th} + sgn_b sum_{j>=1} F_j e^{-i th},
// P = E G, H_i = (1/L) sum_l P(l) e^{-i th_i}; sgn = -1 except b = 3 (+1).
// Both transforms are radix-2 FFTs of length L (a power of two) in shared
// memory: the modes are placed at +j and (times sgn) at L - j.
template <class T>
__global__ void smc_fs_x_kernel(const typename C2<T>::type* __restrict__ Fv, const T* __restrict__ E,
                                int Nk, int Mz, int L, const typename C2<T>::type* __restrict__ tw,
                                typename C2<T>::type* __restrict__ Hv) {
  using CT = typename C2<T>::type;
  extern __shared__ unsigned char smraw[];
  CT* P = reinterpret_cast<CT*>(smraw);    // L
  CT* W = P + L;                           // L/2 twiddles
  const int s = blockIdx.x, b = blockIdx.y, tid = threadIdx.x, nt = blockDim.x;
  const T sgn = (b == 3) ? (T)1 : (T)-1;
  const int logL = ilog2_pow2(L);
  for (int i = tid; i < (L >> 1); i += nt) W[i] = tw[i];
  for (int i = tid; i < L; i += nt) { P[i].x = (T)0; P[i].y = (T)0; }
  __syncthreads();
  for (int j = tid; j < Nk; j += nt) {
    const CT f = Fv[((long long)b * Nk + j) * Mz + s];
    P[j] = f;
    if (j > 0) { P[L - j].x = sgn * f.x; P[L - j].y = sgn * f.y; }
  }
  __syncthreads();
  cta_fft(P, L, logL, W, +1, tid, nt);
  for (int l = tid; l < L; l += nt) {
    const T e = E[(long long)l * Mz + s];
    P[l].x *= e;
    P[l].y *= e;
  }
  __syncthreads();
  cta_fft(P, L, logL, W, -1, tid, nt);
  const T invL = (T)1 / (T)L;
  for (int i = tid; i < Nk; i += nt) {
    CT o;
    o.x = P[i].x * invL;
    o.y = P[i].y * invL;
    Hv[((long long)b * Nk + i) * Mz + s] = o;
  }
}

// out[k][p] = D2Zi (H0 + H1) + Zi (2k^2 H2 - k^2 H0) - 4k DZi H3 ; tau rows
// v(0) = V[0].v, v(1) = V[N-1].v (FP64).  One warp per output, lanes over s.
template <class T>
__global__ void smc_fs_out_kernel(const typename C2<T>::type* __restrict__ Hv, const T* __restrict__ Zi,
                                  const T* __restrict__ D2Zi, const T* __restrict__ DZi,
                                  const double2* __restrict__ v, const double* __restrict__ V,
                                  const double* __restrict__ kx, int Nk, int N, int Mz,
                                  double2* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const long long o = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (o >= (long long)Nk * N) return;
  const int k = (int)(o / N), p = (int)(o % N);
  if (p >= N - 2) {
    const double* Vr = V + (p == N - 2 ? 0 : (long long)(N - 1) * N);
    const double2* vk = v + (long long)k * N;
    double sr = 0, si = 0;
    for (int m = lane; m < N; m += 32) { sr += vk[m].x * Vr[m]; si += vk[m].y * Vr[m]; }
    for (int d = 16; d > 0; d >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, d);
      si += __shfl_xor_sync(0xffffffffu, si, d);
    }
    if (lane == 0) out[o] = make_double2(sr, si);
    return;
  }
  const long long KM = (long long)Nk * Mz;
  const typename C2<T>::type* H0 = Hv + (long long)k * Mz;
  const typename C2<T>::type* H1 = H0 + KM;
  const typename C2<T>::type* H2 = H1 + KM;
  const typename C2<T>::type* H3 = H2 + KM;
  const T* a = D2Zi + (long long)p * Mz;
  const T* z = Zi + (long long)p * Mz;
  const T* dd = DZi + (long long)p * Mz;
  const double kk = kx[k];
  const T k2 = (T)(kk * kk);
  T ar = 0, ai = 0, br = 0, bi = 0, cr = 0, ci = 0;
  for (int q = lane; q < Mz; q += 32) {
    const T as = a[q], zs = z[q], ds = dd[q];
    const typename C2<T>::type h0 = H0[q], h1 = H1[q], h2 = H2[q], h3 = H3[q];
    ar += as * (h0.x + h1.x);
    ai += as * (h0.y + h1.y);
    br += zs * ((T)2 * k2 * h2.x - k2 * h0.x);
    bi += zs * ((T)2 * k2 * h2.y - k2 * h0.y);
    cr += ds * h3.x;
    ci += ds * h3.y;
  }
  for (int d = 16; d > 0; d >>= 1) {
    ar += __shfl_xor_sync(0xffffffffu, ar, d);
    ai += __shfl_xor_sync(0xffffffffu, ai, d);
    br += __shfl_xor_sync(0xffffffffu, br, d);
    bi += __shfl_xor_sync(0xffffffffu, bi, d);
    cr += __shfl_xor_sync(0xffffffffu, cr, d);
    ci += __shfl_xor_sync(0xffffffffu, ci, d);
  }
  if (lane == 0) {
    const double r = (double)ar + (double)br - 4.0 * kk * (double)cr;
    const double im = (double)ai + (double)bi - 4.0 * kk * (double)ci;
    out[o] = make_double2(r, im);
  }
}

__global__ void smc_to_float2_kernel(const double2* __restrict__ in, float2* __restrict__ out,
                                     long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_float2((float)in[i].x, (float)in[i].y);
}

template <class T>
void fused_schur_matvec_t(const Ctx& c, const FusedSchur<T>& op, const T* E, const double2* v,
                          double2* out, void* Fv, void* Hv) {
  using CT = typename C2<T>::type;
  const long long nf = 4LL * op.Nk * op.Mz;
  const CT* vin;
  if (std::is_same<T, float>::value) {
    // one FP64 -> FP32 conversion of the Krylov vector (the FP64 pipe
    // issues conversions; doing it once keeps the operator on FP32 units)
    float2* v32 = reinterpret_cast<float2*>(op.vbuf);
    const long long nv = (long long)op.Nk * op.N;
    smc_to_float2_kernel<<<ceil_div(nv, 256), 256, 0, c.s>>>(v, v32, nv);
    SMC_LAUNCH_CHECK(c);
    vin = reinterpret_cast<const CT*>(v32);
  } else {
    vin = reinterpret_cast<const CT*>(v);
  }
  smc_fs_fwd_kernel<T><<<ceil_div(nf, 8), 256, 0, c.s>>>(vin, op.Zf, op.Z1, op.Z2, op.Z3, op.kx, op.Nk,
                                                        op.N, op.Mz, (CT*)Fv);
  SMC_LAUNCH_CHECK(c);
  dim3 g2(op.Mz, 4);
  size_t sm = (size_t)(op.L + op.L / 2) * sizeof(CT);
  allow_max_smem((const void*)smc_fs_x_kernel<T>);
  smc_fs_x_kernel<T><<<g2, 128, sm, c.s>>>((const CT*)Fv, E, op.Nk, op.Mz, op.L, (const CT*)op.tw,
                                          (CT*)Hv);
  SMC_LAUNCH_CHECK(c);
  const long long no = (long long)op.Nk * op.N;
  smc_fs_out_kernel<T><<<ceil_div(no, 8), 256, 0, c.s>>>((const CT*)Hv, op.Zi, op.D2Zi, op.DZi, v, op.V,
                                                        op.kx, op.Nk, op.N, op.Mz, out);
  SMC_LAUNCH_CHECK(c);
}

void fused_schur_matvec(const Ctx& c, const FusedSchur<double>& op, const double* E,
                        const double2* v, double2* out, void* Fv, void* Hv) {
  fused_schur_matvec_t<double>(c, op, E, v, out, Fv, Hv);
}
void fused_schur_matvec(const Ctx& c, const FusedSchur<float>& op, const float* E,
                        const double2* v, double2* out, void* Fv, void* Hv) {
  fused_schur_matvec_t<float>(c, op, E, v, out, Fv, Hv);
}

// ----------------------------------------------------- temperature matvec
// X0[k][j] = i k (V v_k)[j], X1[k][j] = (VD v_k)[j]; one warp per (k, j)
template <class T>
__global__ void smc_ft_zsynth_kernel(const double2* __restrict__ v, const T* __restrict__ Vt,
                                     const T* __restrict__ VDt, const double* __restrict__ kx, int Nk,
                                     int N, typename C2<T>::type* __restrict__ X) {
  using CT = typename C2<T>::type;
  const int lane = threadIdx.x & 31;
  const long long o = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (o >= (long long)Nk * N) return;
  const int k = (int)(o / N), j = (int)(o % N);
  const T* a = Vt + (long long)j * N;
  const T* d = VDt + (long long)j * N;
  const double2* vk = v + (long long)k * N;
  T ar = 0, ai = 0, dr = 0, di = 0;
  for (int q = lane; q < N; q += 32) {
    const double2 x = vk[q];
    const T xr = (T)x.x, xi = (T)x.y;
    ar += a[q] * xr;
    ai += a[q] * xi;
    dr += d[q] * xr;
    di += d[q] * xi;
  }
  for (int s = 16; s > 0; s >>= 1) {
    ar += __shfl_xor_sync(0xffffffffu, ar, s);
    ai += __shfl_xor_sync(0xffffffffu, ai, s);
    dr += __shfl_xor_sync(0xffffffffu, dr, s);
    di += __shfl_xor_sync(0xffffffffu, di, s);
  }
  if (lane == 0) {
    const T kk = (T)kx[k];
    CT o0, o1;
    o0.x = -kk * ai;      // i k (ar + i ai)
    o0.y = kk * ar;
    o1.x = dr;
    o1.y = di;
    X[(long long)k * N + j] = o0;
    X[(long long)(Nk + k) * N + j] = o1;
  }
}

// per z-column j: vx, vz on the Np padded points, prod = -(ux vx + uz vz),
// A[k][j] = (1/Np) sum_i prod_i e^{-2 pi i k i/Np}
template <class T>
__global__ void smc_ft_x_kernel(const typename C2<T>::type* __restrict__ X, const T* __restrict__ ux,
                                const T* __restrict__ uz, const typename C2<T>::type* __restrict__ tw,
                                int Nk, int N, int Np, typename C2<T>::type* __restrict__ A) {
  using CT = typename C2<T>::type;
  extern __shared__ unsigned char smraw[];
  CT* xa = reinterpret_cast<CT*>(smraw);  // Nk
  CT* xb = xa + Nk;                        // Nk
  CT* W = xb + Nk;                         // Np twiddles
  T* P = reinterpret_cast<T*>(W + Np);    // Np
  const int j = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  for (int k = tid; k < Nk; k += nt) {
    xa[k] = X[(long long)k * N + j];
    xb[k] = X[(long long)(Nk + k) * N + j];
  }
  for (int i = tid; i < Np; i += nt) W[i] = tw[i];
  __syncthreads();
  for (int i = tid; i < Np; i += nt) {
    T a = xa[0].x, b = xb[0].x;
    int idx = 0;
    for (int k = 1; k < Nk; ++k) {
      idx += i;
      if (idx >= Np) idx -= Np;
      const CT t = W[idx];
      const T wk = (2 * k == Np) ? (T)1 : (T)2;
      a += wk * (xa[k].x * t.x - xa[k].y * t.y);
      b += wk * (xb[k].x * t.x - xb[k].y * t.y);
    }
    const long long e = (long long)i * N + j;
    P[i] = -(ux[e] * a + uz[e] * b);
  }
  __syncthreads();
  const T inv = (T)1 / (T)Np;
  for (int k = tid; k < Nk; k += nt) {
    T sr = 0, si = 0;
    int idx = 0;
    for (int i = 0; i < Np; ++i) {
      const CT t = W[idx];
      sr += P[i] * t.x;
      si -= P[i] * t.y;
      idx += k;
      if (idx >= Np) idx -= Np;
    }
    CT o;
    o.x = sr * inv;
    o.y = si * inv;
    A[(long long)k * N + j] = o;
  }
}

// out = a0 v - (D2 v - k^2 v) - Vi A ; tau rows v(0), v(1); one warp per (k, n)
template <class T>
__global__ void smc_ft_out_kernel(const double2* __restrict__ v, const typename C2<T>::type* __restrict__ A,
                                  const T* __restrict__ D2t, const T* __restrict__ Vit,
                                  const double* __restrict__ V, const double* __restrict__ kx, double a0,
                                  int Nk, int N, double2* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const long long o = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (o >= (long long)Nk * N) return;
  const int k = (int)(o / N), n = (int)(o % N);
  const double2* vk = v + (long long)k * N;
  if (n >= N - 2) {
    const double* Vr = V + (n == N - 2 ? 0 : (long long)(N - 1) * N);
    double sr = 0, si = 0;
    for (int m = lane; m < N; m += 32) { sr += vk[m].x * Vr[m]; si += vk[m].y * Vr[m]; }
    for (int d = 16; d > 0; d >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, d);
      si += __shfl_xor_sync(0xffffffffu, si, d);
    }
    if (lane == 0) out[o] = make_double2(sr, si);
    return;
  }
  const T* dr = D2t + (long long)n * N;
  const T* vi = Vit + (long long)n * N;
  const typename C2<T>::type* Ak = A + (long long)k * N;
  T lr = 0, li = 0, ar = 0, ai = 0;
  for (int m = lane; m < N; m += 32) {
    lr += dr[m] * (T)vk[m].x;
    li += dr[m] * (T)vk[m].y;
    ar += vi[m] * Ak[m].x;
    ai += vi[m] * Ak[m].y;
  }
  for (int d = 16; d > 0; d >>= 1) {
    lr += __shfl_xor_sync(0xffffffffu, lr, d);
    li += __shfl_xor_sync(0xffffffffu, li, d);
    ar += __shfl_xor_sync(0xffffffffu, ar, d);
    ai += __shfl_xor_sync(0xffffffffu, ai, d);
  }
  if (lane == 0) {
    const double k2 = kx[k] * kx[k];
    const double2 vn = vk[n];
    const double Lr = (double)lr - k2 * vn.x, Li = (double)li - k2 * vn.y;
    out[o] = make_double2((a0 * vn.x - Lr) - (double)ar, (a0 * vn.y - Li) - (double)ai);
  }
}

template <class T>
void fused_theta_matvec_t(const Ctx& c, const FusedTheta<T>& op, const T* ux, const T* uz,
                          double a0, const double2* v, double2* out, void* X, void* A) {
  using CT = typename C2<T>::type;
  const long long no = (long long)op.Nk * op.N;
  smc_ft_zsynth_kernel<T><<<ceil_div(no, 8), 256, 0, c.s>>>(v, op.V, op.VD, op.kx, op.Nk, op.N, (CT*)X);
  SMC_LAUNCH_CHECK(c);
  size_t sm = (size_t)(2 * op.Nk + op.Np) * sizeof(CT) + op.Np * sizeof(T);
  allow_max_smem((const void*)smc_ft_x_kernel<T>);
  smc_ft_x_kernel<T><<<op.N, 128, sm, c.s>>>((const CT*)X, ux, uz, (const CT*)op.tw, op.Nk, op.N,
                                            op.Np, (CT*)A);
  SMC_LAUNCH_CHECK(c);
  smc_ft_out_kernel<T><<<ceil_div(no, 8), 256, 0, c.s>>>(v, (const CT*)A, op.D2, op.Vi, op.V64, op.kx,
                                                         a0, op.Nk, op.N, out);
  SMC_LAUNCH_CHECK(c);
}

void fused_theta_matvec(const Ctx& c, const FusedTheta<double>& op, const double* ux,
                        const double* uz, double a0, const double2* v, double2* out, void* X,
                        void* A) {
  fused_theta_matvec_t<double>(c, op, ux, uz, a0, v, out, X, A);
}
void fused_theta_matvec(const Ctx& c, const FusedTheta<float>& op, const float* ux, const float* uz,
                        double a0, const double2* v, double2* out, void* X, void* A) {
  fused_theta_matvec_t<float>(c, op, ux, uz, a0, v, out, X, A);
}

// ----------------------------------------------------------- CGS2 Arnoldi
// w <- w - V h twice (classical Gram-Schmidt with one reorthogonalisation),
// hout[0..j] = accumulated h, hout[j+1] = ||w||.  Cooperative: every CTA owns
// a contiguous slice of the vectors; 3 grid barriers per call.  part holds
// 2 * G * (j+1) complex partials (two buffers) + G norm partials.
__global__ void __launch_bounds__(256) smc_cgs2_kernel(const double2* __restrict__ Vb, int j,
                                                      long long n, double2* __restrict__ w,
                                                      double2* __restrict__ hout,
                                                      double2* __restrict__ part) {
  cg::grid_group grid = cg::this_grid();
  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long per = (n + G - 1) / G;
  const long long lo = b * per, hi = min(n, lo + per);
  const int m = j + 1;
  __shared__ double2 h[96], hsum[96];
  __shared__ double nred[8];
  for (int i = tid; i < m; i += 256) hsum[i] = make_double2(0.0, 0.0);
  for (int pass = 0; pass < 2; ++pass) {
    double2* pp = part + (size_t)pass * G * m;
    // partial dots: warp per vector i (strided), lanes over the slice
    for (int i = warp; i < m; i += 8) {
      const double2* Vi = Vb + (long long)i * n;
      double sr = 0.0, si = 0.0;
      for (long long t = lo + lane; t < hi; t += 32) {
        double2 a = Vi[t], x = w[t];
        sr += a.x * x.x + a.y * x.y;
        si += a.x * x.y - a.y * x.x;
      }
      for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
        si += __shfl_xor_sync(0xffffffffu, si, o);
      }
      if (lane == 0) pp[(size_t)b * m + i] = make_double2(sr, si);
    }
    grid.sync();
    for (int i = warp; i < m; i += 8) {          // warp per vector, lanes over CTAs
      double sr = 0.0, si = 0.0;
      for (int g = lane; g < G; g += 32) {
        double2 q = pp[(size_t)g * m + i];
        sr += q.x;
        si += q.y;
      }
      for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
        si += __shfl_xor_sync(0xffffffffu, si, o);
      }
      if (lane == 0) {
        h[i] = make_double2(sr, si);
        hsum[i] = cadd(hsum[i], h[i]);
      }
    }
    __syncthreads();
    for (long long t = lo + tid; t < hi; t += 256) {
      double2 x = w[t];
      for (int i = 0; i < m; ++i) x = csub(x, cmul(h[i], Vb[(long long)i * n + t]));
      w[t] = x;
    }
    __syncthreads();
  }
  double s = 0.0;
  for (long long t = lo + tid; t < hi; t += 256) s += w[t].x * w[t].x + w[t].y * w[t].y;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) nred[warp] = s;
  __syncthreads();
  double2* np = part + (size_t)2 * G * m;
  if (tid == 0) {
    double a = 0.0;
    for (int q = 0; q < 8; ++q) a += nred[q];
    np[b] = make_double2(a, 0.0);
  }
  grid.sync();
  if (b == 0) {
    for (int i = tid; i < m; i += 256) hout[i] = hsum[i];
    if (warp == 0) {
      double a = 0.0;
      for (int g = lane; g < G; g += 32) a += np[g].x;
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if (lane == 0) hout[m] = make_double2(sqrt(a), 0.0);
    }
  }
}

void cgs2(const Ctx& c, const double2* V, int j, long long n, double2* w, double2* hout,
          double2* part) {
  if (j + 1 > 96) throw std::runtime_error("cgs2: restart above 95");
  int G = c.num_sms;
  void* args[] = {(void*)&V, (void*)&j, (void*)&n, (void*)&w, (void*)&hout, (void*)&part};
  CoopGuard guard(c.s);
  SMC_CUDA(cudaLaunchCooperativeKernel((void*)smc_cgs2_kernel, dim3(G), dim3(256), args, 0, c.s));
  SMC_LAUNCH_CHECK(c);
}

// ------------------------------------------------ per-k operator GEMV
// out[k][n] = alpha sum_m G[k][n][m] r[k][m]  (G real, row-major per k)
__global__ void smc_kgemv_kernel(const double* __restrict__ G, const double2* __restrict__ r,
                                 double2* __restrict__ out, int Nk, int N, double alpha) {
  const int lane = threadIdx.x & 31;
  const long long o = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (o >= (long long)Nk * N) return;
  const int k = (int)(o / N), n = (int)(o % N);
  const double* g = G + ((long long)k * N + n) * N;
  const double2* rk = r + (long long)k * N;
  double sr = 0.0, si = 0.0;
  for (int m = lane; m < N; m += 32) {
    const double w = g[m];
    sr += w * rk[m].x;
    si += w * rk[m].y;
  }
  for (int d = 16; d > 0; d >>= 1) {
    sr += __shfl_xor_sync(0xffffffffu, sr, d);
    si += __shfl_xor_sync(0xffffffffu, si, d);
  }
  if (lane == 0) out[o] = make_double2(alpha * sr, alpha * si);
}

void kgemv(const Ctx& c, const double* G, const double2* r, double2* out, int Nk, int N,
           double alpha) {
  const long long no = (long long)Nk * N;
  smc_kgemv_kernel<<<ceil_div(no, 8), 256, 0, c.s>>>(G, r, out, Nk, N, alpha);
  SMC_LAUNCH_CHECK(c);
}

// --------------------------------------------------------- set-up helpers
// C_b = A_b (M x K) . B_b (K x Nc), real, row-major, batch strides
__global__ void smc_rgemm_kernel(const double* __restrict__ A, long long sa, const double* __restrict__ B,
                                 long long sb, double* __restrict__ C, long long sc, int M, int K,
                                 int Nc) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = blockIdx.y;
  const long long bt = blockIdx.z;
  if (col >= Nc) return;
  const double* a = A + bt * sa + (long long)row * K;
  const double* bb = B + bt * sb + col;
  double s = 0.0;
  for (int q = 0; q < K; ++q) s += a[q] * bb[(long long)q * Nc];
  C[bt * sc + (long long)row * Nc + col] = s;
}

void rgemm_batched(const Ctx& c, const double* A, long long sa, const double* B, long long sb,
                   double* C, long long sc, int M, int K, int Nc, int batch) {
  dim3 g(ceil_div(Nc, 128), M, batch);
  smc_rgemm_kernel<<<g, 128, 0, c.s>>>(A, sa, B, sb, C, sc, M, K, Nc);
  SMC_LAUNCH_CHECK(c);
}

__global__ void smc_d2f_kernel(const double* in, float* out, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}

void to_float(const Ctx& c, const double* in, float* out, long long n) {
  smc_d2f_kernel<<<ceil_div(n, 256), 256, 0, c.s>>>(in, out, n);
  SMC_LAUNCH_CHECK(c);
}

}  // namespace smc
