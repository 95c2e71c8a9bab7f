// Coupled variable-viscosity Stokes operator of the FP64 time step.
//
//  * Chebyshev product matrices M_d of the x-modes d of eta
//    (stokes/vv_stokes.py:81-109, stokes/stokes_coupled.py:123-129,158-168).
//  * mult_eta: the one-sided rfft convolution of eta with a spectral field,
//    including the conjugate ("partner") half (stokes/lagged_stokes.py:162-193).
//  * Dense Schur assembly A[i,j] = Lm_i M_{i-j} + C_ij G_j (+ partner half,
//    tau rows) (stokes/stokes_coupled.py:242-289).
//  * The eta(T) pipeline on the padded grid: T clip, viscosity law, eta window
//    with its dead-band and counters (models/coupled_model.py:333-399,
//    physics/eta_bounds.py:360-480).
//  * Batched small GEMMs for operator set-up (the reduced eta(z) operator and
//    the BFBT blocks, stokes/vv_stokes.py:298-307, stokes/bfbt.py:157-182).
#include "smc_internal.cuh"
#include "smc_schur.cuh"

namespace smc {

// ----------------------------------------------------------- M_d matrices
// Md[(d + Nk - 1)][p][q] = 1/2 (a[p-q][p>=q] + a[p+q][p+q<N] + a[q-p][q>=p>0]),
// a = eta_c[d] (d >= 0) or conj(eta_c[-d]) (d < 0); row-major.
__global__ void smc_build_mult_kernel(const double2* __restrict__ eta_c, double2* __restrict__ Md,
                                      int Nk, int N) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  int p = blockIdx.y;
  int di = blockIdx.z;
  if (q >= N) return;
  int d = di - (Nk - 1);
  const double2* a = eta_c + (long long)(d >= 0 ? d : -d) * N;
  const bool cj = d < 0;
  double sr = 0.0, si = 0.0;
  if (p >= q) { double2 v = a[p - q]; sr += v.x; si += v.y; }
  if (p + q < N) { double2 v = a[p + q]; sr += v.x; si += v.y; }
  if (p > 0 && q >= p) { double2 v = a[q - p]; sr += v.x; si += v.y; }
  if (cj) si = -si;
  Md[((long long)di * N + p) * N + q] = make_double2(0.5 * sr, 0.5 * si);
}

void build_mult_mats(const Ctx& c, const double2* eta_c, double2* Md, int Nk, int N) {
  dim3 grd(ceil_div(N, 128), N, 2 * Nk - 1);
  smc_build_mult_kernel<<<grd, 128, 0, c.s>>>(eta_c, Md, Nk, N);
  SMC_LAUNCH_CHECK(c);
}

// ----------------------------------------------------------------- mult_eta
// out[i][p] = sum_j (M_{i-j} f_j)[p] + sgn sum_{m=1}^{Nk-1-i} (M_{i+m} f_m)[p]
// one warp per output (i, p); lanes split the contraction index q.
__global__ void smc_mult_eta_kernel(const double2* __restrict__ Md, const double2* __restrict__ f,
                                    double2* __restrict__ out, int Nk, int N, double sgn) {
  const int lane = threadIdx.x & 31;
  const long long o = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (o >= (long long)Nk * N) return;
  const int i = (int)(o / N), p = (int)(o % N);
  double ar = 0.0, ai = 0.0;
  for (int j = 0; j < Nk; ++j) {
    const double2* Mrow = Md + ((long long)(i - j + Nk - 1) * N + p) * N;
    const double2* fj = f + (long long)j * N;
    for (int q = lane; q < N; q += 32) {
      double2 m = Mrow[q], v = fj[q];
      ar += m.x * v.x - m.y * v.y;
      ai += m.x * v.y + m.y * v.x;
    }
  }
  if (sgn != 0.0) {
    double br = 0.0, bi = 0.0;
    for (int m = 1; m < Nk - i; ++m) {
      const double2* Mrow = Md + ((long long)(i + m + Nk - 1) * N + p) * N;
      const double2* fm = f + (long long)m * N;
      for (int q = lane; q < N; q += 32) {
        double2 mm = Mrow[q], v = fm[q];
        br += mm.x * v.x - mm.y * v.y;
        bi += mm.x * v.y + mm.y * v.x;
      }
    }
    ar += sgn * br;
    ai += sgn * bi;
  }
  for (int s = 16; s > 0; s >>= 1) {
    ar += __shfl_xor_sync(0xffffffffu, ar, s);
    ai += __shfl_xor_sync(0xffffffffu, ai, s);
  }
  if (lane == 0) out[o] = make_double2(ar, ai);
}

void mult_eta(const Ctx& c, const double2* Md, const double2* f, double2* out, int Nk, int N,
              double sgn, double2* /*partial*/) {
  long long nout = (long long)Nk * N;
  int wpb = 8;
  smc_mult_eta_kernel<<<ceil_div(nout, wpb), 32 * wpb, 0, c.s>>>(Md, f, out, Nk, N, sgn);
  SMC_LAUNCH_CHECK(c);
}

// -------------------------------------------------------- batched small GEMM
// C_b = A_b . B_b (N x N, row-major), each operand real or complex.  32x32
// output tile per CTA, 256 threads, 2x2 outputs per thread.
template <bool AC, bool BC>
__global__ void smc_bgemm_kernel(const void* __restrict__ A, long long sa, const void* __restrict__ B,
                                 long long sb, void* __restrict__ C, long long sc, int N,
                                 double alpha) {
  constexpr bool CC = AC || BC;
  __shared__ double2 As[32][33];
  __shared__ double2 Bs[32][33];
  const long long bt = blockIdx.z;
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double2 acc[2][2] = {{{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}};
  for (int k0 = 0; k0 < N; k0 += 32) {
    for (int t = threadIdx.x; t < 1024; t += 256) {
      int rr = t / 32, kk = t % 32;
      int gr = r0 + rr, gk = k0 + kk;
      double2 va = make_double2(0.0, 0.0), vb = make_double2(0.0, 0.0);
      if (gr < N && gk < N) {
        long long ia = bt * sa + (long long)gr * N + gk;
        va = AC ? ((const double2*)A)[ia] : make_double2(((const double*)A)[ia], 0.0);
      }
      int gk2 = k0 + rr, gc = c0 + kk;
      if (gk2 < N && gc < N) {
        long long ib = bt * sb + (long long)gk2 * N + gc;
        vb = BC ? ((const double2*)B)[ib] : make_double2(((const double*)B)[ib], 0.0);
      }
      As[rr][kk] = va;
      Bs[rr][kk] = vb;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < 32; ++kk) {
      double2 a0 = As[ty * 2][kk], a1 = As[ty * 2 + 1][kk];
      double2 b0 = Bs[kk][tx * 2], b1 = Bs[kk][tx * 2 + 1];
      if (CC) {
        acc[0][0] = cadd(acc[0][0], cmul(a0, b0));
        acc[0][1] = cadd(acc[0][1], cmul(a0, b1));
        acc[1][0] = cadd(acc[1][0], cmul(a1, b0));
        acc[1][1] = cadd(acc[1][1], cmul(a1, b1));
      } else {
        acc[0][0].x += a0.x * b0.x;
        acc[0][1].x += a0.x * b1.x;
        acc[1][0].x += a1.x * b0.x;
        acc[1][1].x += a1.x * b1.x;
      }
    }
    __syncthreads();
  }
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      int gr = r0 + ty * 2 + i, gc = c0 + tx * 2 + j;
      if (gr >= N || gc >= N) continue;
      long long ic = bt * sc + (long long)gr * N + gc;
      if (CC) ((double2*)C)[ic] = cscale(acc[i][j], alpha);
      else ((double*)C)[ic] = alpha * acc[i][j].x;
    }
}

void bgemm(const Ctx& c, bool a_cplx, const void* A, long long sa, bool b_cplx, const void* B,
           long long sb, void* C, long long sc, int N, int batch, double alpha) {
  dim3 grd(ceil_div(N, 32), ceil_div(N, 32), batch);
  if (a_cplx && b_cplx) smc_bgemm_kernel<true, true><<<grd, 256, 0, c.s>>>(A, sa, B, sb, C, sc, N, alpha);
  else if (a_cplx) smc_bgemm_kernel<true, false><<<grd, 256, 0, c.s>>>(A, sa, B, sb, C, sc, N, alpha);
  else if (b_cplx) smc_bgemm_kernel<false, true><<<grd, 256, 0, c.s>>>(A, sa, B, sb, C, sc, N, alpha);
  else smc_bgemm_kernel<false, false><<<grd, 256, 0, c.s>>>(A, sa, B, sb, C, sc, N, alpha);
  SMC_LAUNCH_CHECK(c);
}

// ------------------------------------------------------------ Schur assembly
// Block (i, j) of the dense Schur matrix, written column-major into A (n x n):
//   B = D2M_d - ki^2 M_d + T G_j,
//   T = 2kj^2 D2M_d + 2ki^2 MD2_d - 4 ki kj DMD_d
// plus, for j >= 1 and i + j < Nk, the partner half with sign -1 and the
// cross term flipped (shift i + j).  Tau rows N-2, N-1 are the v(0), v(1)
// rows on the diagonal block and zero elsewhere.
__global__ void smc_schur_block_kernel(const double2* __restrict__ Md, const double2* __restrict__ P1,
                                       const double2* __restrict__ P2, const double2* __restrict__ P3,
                                       const double* __restrict__ G, const double* __restrict__ V,
                                       const double* __restrict__ kx, double2* __restrict__ A,
                                       int Nk, int N) {
  __shared__ double2 Ts[32][33];
  __shared__ double Gs[32][33];
  const int blk = blockIdx.z;
  const int i = blk / Nk, j = blk % Nk;
  const int p0 = blockIdx.y * 32, r0 = blockIdx.x * 32;
  const long long n = (long long)Nk * N;
  const double ki = kx[i], kj = kx[j];
  const int dd = i - j + Nk - 1;
  const bool part = (j >= 1) && (i + j < Nk);
  const int dp = i + j + Nk - 1;
  const long long NN = (long long)N * N;
  const double cd1 = 2.0 * kj * kj, cd2 = 2.0 * ki * ki, cd3 = -4.0 * ki * kj;
  const int tp = threadIdx.x % 16, tr = threadIdx.x / 16;   // p fastest for the column-major store
  double2 acc[2][2] = {{{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}};
  const double* Gj = G + (long long)j * NN;
  for (int k0 = 0; k0 < N; k0 += 32) {
    for (int t = threadIdx.x; t < 1024; t += 256) {
      int pp = t / 32, kk = t % 32;
      int gp = p0 + pp, gk = k0 + kk;
      double2 tv = make_double2(0.0, 0.0);
      if (gp < N && gk < N) {
        long long e = (long long)gp * N + gk;
        double2 a1 = P1[dd * NN + e], a2 = P2[dd * NN + e], a3 = P3[dd * NN + e];
        tv = make_double2(cd1 * a1.x + cd2 * a2.x + cd3 * a3.x, cd1 * a1.y + cd2 * a2.y + cd3 * a3.y);
        if (part) {
          double2 b1 = P1[dp * NN + e], b2 = P2[dp * NN + e], b3 = P3[dp * NN + e];
          tv.x -= cd1 * b1.x + cd2 * b2.x - cd3 * b3.x;
          tv.y -= cd1 * b1.y + cd2 * b2.y - cd3 * b3.y;
        }
      }
      Ts[pp][kk] = tv;
      int gk2 = k0 + pp, gr = r0 + kk;
      Gs[pp][kk] = (gk2 < N && gr < N) ? Gj[(long long)gk2 * N + gr] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < 32; ++kk) {
      double2 t0 = Ts[tp * 2][kk], t1 = Ts[tp * 2 + 1][kk];
      double g0 = Gs[kk][tr * 2], g1 = Gs[kk][tr * 2 + 1];
      acc[0][0].x += t0.x * g0; acc[0][0].y += t0.y * g0;
      acc[0][1].x += t0.x * g1; acc[0][1].y += t0.y * g1;
      acc[1][0].x += t1.x * g0; acc[1][0].y += t1.y * g0;
      acc[1][1].x += t1.x * g1; acc[1][1].y += t1.y * g1;
    }
    __syncthreads();
  }
  for (int b = 0; b < 2; ++b)
    for (int a = 0; a < 2; ++a) {
      int gp = p0 + tp * 2 + a, gr = r0 + tr * 2 + b;
      if (gp >= N || gr >= N) continue;
      long long e = (long long)gp * N + gr;
      double2 v;
      if (gp >= N - 2) {
        double bc = (i == j) ? V[(gp == N - 2 ? 0 : (long long)(N - 1) * N) + gr] : 0.0;
        v = make_double2(bc, 0.0);
      } else {
        double2 m1 = P1[dd * NN + e], m0 = Md[dd * NN + e];
        v = make_double2(m1.x - ki * ki * m0.x + acc[a][b].x, m1.y - ki * ki * m0.y + acc[a][b].y);
        if (part) {
          double2 q1 = P1[dp * NN + e], q0 = Md[dp * NN + e];
          v.x -= q1.x - ki * ki * q0.x;
          v.y -= q1.y - ki * ki * q0.y;
        }
      }
      A[((long long)i * N + gp) + ((long long)j * N + gr) * n] = v;
    }
}

void assemble_schur(const Ctx& c, const double2* Md, const double* D, const double* D2,
                    const double* G, const double* V, const double* kx, double2* A, int Nk,
                    int N, double2* work) {
  const long long NN = (long long)N * N;
  const int nd = 2 * Nk - 1;
  double2* P1 = work;              // D2 M_d
  double2* P2 = P1 + nd * NN;      // M_d D2
  double2* P3 = P2 + nd * NN;      // D M_d D
  double2* T = P3 + nd * NN;       // M_d D (scratch)
  bgemm(c, false, D2, 0, true, Md, NN, P1, NN, N, nd, 1.0);
  bgemm(c, true, Md, NN, false, D2, 0, P2, NN, N, nd, 1.0);
  bgemm(c, true, Md, NN, false, D, 0, T, NN, N, nd, 1.0);
  bgemm(c, false, D, 0, true, T, NN, P3, NN, N, nd, 1.0);
  dim3 grd(ceil_div(N, 32), ceil_div(N, 32), Nk * Nk);
  smc_schur_block_kernel<<<grd, 256, 0, c.s>>>(Md, P1, P2, P3, G, V, kx, A, Nk, N);
  SMC_LAUNCH_CHECK(c);
}

// ------------------------------------------------------------- eta pipeline
// T = 1 - z_j + th on the padded grid; statistics of the reference's
// counters; eta = law(clip(T, 0, 2)); the window: hard (counted only, the
// clamp is applied by smc_eta_clip_kernel iff any point is outside the
// dead-band window) or smooth (C^2 clamp in ln eta, always applied).
__global__ void smc_eta_law_kernel(const double* __restrict__ th, const double* __restrict__ z,
                                   int N, long long npts, EtaLaw law, double* __restrict__ eta,
                                   double* __restrict__ part) {
  double tmin = INFINITY, tmax = -INFINITY;
  double c_oor = 0, c_clipT = 0, c_clip = 0, c_band = 0;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < npts;
       idx += (long long)gridDim.x * blockDim.x) {
    int j = (int)(idx % N);
    double T = law.z_mode == 1 ? th[idx] : 1.0 - z[j] + th[idx];
    tmin = fmin(tmin, T);
    tmax = fmax(tmax, T);
    if (T < 0.0 || T > 1.0) c_oor += 1.0;
    if (T < 0.0 || T > 2.0) c_clipT += 1.0;
    double Tc = fmin(fmax(T, 0.0), 2.0);
    double e;
    if (law.pvV > 0.0)      // pV(L), physics/arrhenius.py:283-327, in the reference's order
      e = exp((-law.pvE * Tc) / (law.Ts * (Tc + law.Ts)) + law.pvV * (1.0 - z[j]) / (Tc + law.Ts));
    else if (law.Ts > 0.0) e = exp(-law.L * (1.0 + law.Ts) * Tc / (Tc + law.Ts));
    else e = exp(-law.L * Tc);
    if (e < law.lo_eff || e > law.hi_eff) c_clip += 1.0;
    if (law.w > 0.0) {
      double y = log(e);
      if ((y > law.ylo && y < law.ylo + law.w) || (y > law.yhi - law.w && y < law.yhi)) c_band += 1.0;
      double t1 = fmin(fmax((y - law.ylo) / law.w, 0.0), 1.0);
      double Y = law.ylo + (y - law.ylo) * (t1 * t1 * t1 * (t1 * (6.0 * t1 - 15.0) + 10.0));
      double t2 = fmin(fmax((law.yhi - Y) / law.w, 0.0), 1.0);
      double yo = law.yhi - (law.yhi - Y) * (t2 * t2 * t2 * (t2 * (6.0 * t2 - 15.0) + 10.0));
      e = exp(yo);
    }
    eta[idx] = e;
  }
  // reduce (fmin via max of negatives)
  double r_nmin = -INFINITY, r_max = -INFINITY;
  {
    double v = -tmin;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    r_nmin = v;
    v = tmax;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    r_max = v;
  }
  double s[4] = {c_oor, c_clipT, c_clip, c_band};
  for (int q = 0; q < 4; ++q)
    for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
  __shared__ double ws[8][6];
  int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    ws[w][0] = r_nmin; ws[w][1] = r_max;
    for (int q = 0; q < 4; ++q) ws[w][2 + q] = s[q];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a0 = -INFINITY, a1 = -INFINITY, a[4] = {0, 0, 0, 0};
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
      a0 = fmax(a0, ws[q][0]); a1 = fmax(a1, ws[q][1]);
      for (int t = 0; t < 4; ++t) a[t] += ws[q][2 + t];
    }
    double* o = part + 6LL * blockIdx.x;
    o[0] = a0; o[1] = a1; o[2] = a[0]; o[3] = a[1]; o[4] = a[2]; o[5] = a[3];
  }
}

// one warp: lanes stride over the per-CTA partials (maxima, and counts that
// are exact in any summation order)
__device__ __forceinline__ void eta_stats_reduce(const double* part, int np, double* dst) {
  const int lane = threadIdx.x & 31;
  double a0 = -INFINITY, a1 = -INFINITY, a[4] = {0, 0, 0, 0};
  for (int b = lane; b < np; b += 32) {
    const double* o = part + 6LL * b;
    a0 = fmax(a0, o[0]); a1 = fmax(a1, o[1]);
    for (int t = 0; t < 4; ++t) a[t] += o[2 + t];
  }
  for (int d = 16; d > 0; d >>= 1) {
    a0 = fmax(a0, __shfl_xor_sync(0xffffffffu, a0, d));
    a1 = fmax(a1, __shfl_xor_sync(0xffffffffu, a1, d));
    for (int t = 0; t < 4; ++t) a[t] += __shfl_xor_sync(0xffffffffu, a[t], d);
  }
  if (lane == 0) {
    dst[0] = -a0; dst[1] = a1;
    for (int t = 0; t < 4; ++t) dst[2 + t] = a[t];
  }
}
__global__ void smc_eta_stats_final_kernel(const double* part, int np, double* dst) {
  if (threadIdx.x < 32) eta_stats_reduce(part, np, dst);
}

void eta_law(const Ctx& c, const double* th, const double* z, int N, long long npts,
             const EtaLaw& law, double* eta, double* stats, double* scratch) {
  int nb = (int)std::min<long long>(120, (npts + 255) / 256);
  if (nb < 1) nb = 1;
  smc_eta_law_kernel<<<nb, 256, 0, c.s>>>(th, z, N, npts, law, eta, scratch);
  SMC_LAUNCH_CHECK(c);
  if (!stats) return;
  smc_eta_stats_final_kernel<<<1, 32, 0, c.s>>>(scratch, nb, stats);
  SMC_LAUNCH_CHECK(c);
}

// the window applied to one value: the smooth C^2 clamp in ln eta (counting
// the values strictly inside a band) or the hard clamp np.clip(eta, lo, hi)
__device__ __forceinline__ double eta_window_value(double e, const EtaLaw& law, double& c_band) {
  if (law.w > 0.0) {
    double y = log(e);
    if ((y > law.ylo && y < law.ylo + law.w) || (y > law.yhi - law.w && y < law.yhi)) c_band += 1.0;
    double t1 = fmin(fmax((y - law.ylo) / law.w, 0.0), 1.0);
    double Y = law.ylo + (y - law.ylo) * (t1 * t1 * t1 * (t1 * (6.0 * t1 - 15.0) + 10.0));
    double t2 = fmin(fmax((law.yhi - Y) / law.w, 0.0), 1.0);
    double yo = law.yhi - (law.yhi - Y) * (t2 * t2 * t2 * (t2 * (6.0 * t2 - 15.0) + 10.0));
    return exp(yo);
  }
  return fmin(fmax(e, law.lo), law.hi);
}

// the window applied to an existing field (hard clamp, or smooth clamp with
// counting) -- the padded-law clamp and the post-truncation guard
__global__ void smc_eta_window_kernel(double* __restrict__ eta, long long npts, EtaLaw law,
                                      int count_only, double* __restrict__ part) {
  double c_clip = 0, c_band = 0;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < npts;
       idx += (long long)gridDim.x * blockDim.x) {
    double e = eta[idx];
    if (e < law.lo_eff || e > law.hi_eff) c_clip += 1.0;
    if (count_only) continue;
    eta[idx] = eta_window_value(e, law, c_band);
  }
  for (int o = 16; o > 0; o >>= 1) {
    c_clip += __shfl_xor_sync(0xffffffffu, c_clip, o);
    c_band += __shfl_xor_sync(0xffffffffu, c_band, o);
  }
  __shared__ double ws[8][2];
  if ((threadIdx.x & 31) == 0) { ws[threadIdx.x >> 5][0] = c_clip; ws[threadIdx.x >> 5][1] = c_band; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { a += ws[q][0]; b += ws[q][1]; }
    part[2LL * blockIdx.x] = a;
    part[2LL * blockIdx.x + 1] = b;
  }
}

__global__ void smc_sum2_final_kernel(const double* part, int np, double* dst) {
  if (threadIdx.x != 0) return;
  double a = 0, b = 0;
  for (int i = 0; i < np; ++i) { a += part[2 * i]; b += part[2 * i + 1]; }
  dst[0] = a;
  dst[1] = b;
}

void eta_window(const Ctx& c, double* eta, long long npts, const EtaLaw& law, int count_only,
                double* counts, double* scratch) {
  int nb = (int)std::min<long long>(120, (npts + 255) / 256);
  if (nb < 1) nb = 1;
  smc_eta_window_kernel<<<nb, 256, 0, c.s>>>(eta, npts, law, count_only, scratch);
  SMC_LAUNCH_CHECK(c);
  smc_sum2_final_kernel<<<1, 32, 0, c.s>>>(scratch, nb, counts);
  SMC_LAUNCH_CHECK(c);
}

// min over a field (the positivity test of the guard) and the pointwise
// relative drift max |eta - eta_lag| / max(|eta_lag|, 1e-300)
__global__ void smc_min_drift_kernel(const double* __restrict__ eta, const double* __restrict__ lag,
                                     long long n, double* __restrict__ part) {
  double mn = INFINITY, dr = 0.0;
  bool nan_seen = false;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double e = eta[i];
    if (e != e) nan_seen = true;
    mn = fmin(mn, e);
    if (lag) {
      double l = lag[i];
      double v = fabs(e - l) / fmax(fabs(l), 1e-300);
      if (v != v) nan_seen = true;
      dr = fmax(dr, v);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    dr = fmax(dr, __shfl_xor_sync(0xffffffffu, dr, o));
  }
  __shared__ double ws[8][2];
  int any_nan = __syncthreads_or(nan_seen);
  if ((threadIdx.x & 31) == 0) { ws[threadIdx.x >> 5][0] = mn; ws[threadIdx.x >> 5][1] = dr; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = INFINITY, b = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { a = fmin(a, ws[q][0]); b = fmax(b, ws[q][1]); }
    part[2LL * blockIdx.x] = any_nan ? NAN : a;
    part[2LL * blockIdx.x + 1] = any_nan ? NAN : b;
  }
}

// one warp: min and max over the per-CTA partials, NaN if any partial is NaN
__global__ void smc_min_drift_final_kernel(const double* part, int np, double* dst) {
  const int lane = threadIdx.x & 31;
  if (threadIdx.x >= 32) return;
  double a = INFINITY, b = 0.0;
  bool nan_seen = false;
  for (int i = lane; i < np; i += 32) {
    double x = part[2 * i], y = part[2 * i + 1];
    if (x != x || y != y) nan_seen = true;
    a = fmin(a, x);
    b = fmax(b, y);
  }
  for (int d = 16; d > 0; d >>= 1) {
    a = fmin(a, __shfl_xor_sync(0xffffffffu, a, d));
    b = fmax(b, __shfl_xor_sync(0xffffffffu, b, d));
  }
  nan_seen = __any_sync(0xffffffffu, nan_seen);
  if (lane == 0) {
    dst[0] = nan_seen ? NAN : a;
    dst[1] = nan_seen ? NAN : b;
  }
}

void min_and_drift(const Ctx& c, const double* eta, const double* lag, long long n, double* dst,
                   double* scratch) {
  int nb = (int)std::min<long long>(120, (n + 255) / 256);
  if (nb < 1) nb = 1;
  smc_min_drift_kernel<<<nb, 256, 0, c.s>>>(eta, lag, n, scratch);
  SMC_LAUNCH_CHECK(c);
  if (!dst) return;
  smc_min_drift_final_kernel<<<1, 32, 0, c.s>>>(scratch, nb, dst);
  SMC_LAUNCH_CHECK(c);
}

// ------------------------------------------- the eta counters on the device
// std::max(a, b) of the host: b only when a < b (a NaN b is never taken)
__device__ __forceinline__ double host_max(double a, double b) { return (a < b) ? b : a; }

// block sum of one value per thread (256 threads); thread 0 returns it
__device__ __forceinline__ double block_sum256(double v, double* ws) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += ws[q];
  return s;
}

__global__ void smc_eta_stats_apply_kernel(const double* __restrict__ part, int np,
                                           double* __restrict__ eta, long long npts, EtaLaw law,
                                           EtaCtrDev* __restrict__ ctr) {
  // every CTA reduces the law kernel's partials itself (the same values)
  __shared__ double st[6];
  if (threadIdx.x < 32) eta_stats_reduce(part, np, st);
  __syncthreads();
  const double clip = st[4];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const double tmin = st[0], tmax = st[1];
    ctr->max_T_excursion = host_max(ctr->max_T_excursion,
                                    host_max(host_max(0.0 - tmin, tmax - 1.0), 0.0));
    ctr->n_T_out_of_range += (long long)st[2];
    ctr->n_clip_T += (long long)st[3];
    if (law.w > 0.0) {
      ctr->n_clip_eta += (long long)clip;
      ctr->n_smooth_eta += (long long)st[5];
    } else if (clip > 0.0) {
      ctr->n_clip_eta += (long long)clip;
    }
  }
  if (law.w > 0.0 || !(clip > 0.0)) return;     // smooth: already applied by the law
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < npts;
       idx += (long long)gridDim.x * blockDim.x)
    eta[idx] = fmin(fmax(eta[idx], law.lo), law.hi);
}

void eta_stats_apply(const Ctx& c, const double* part, double* eta, long long npts,
                     const EtaLaw& law, EtaCtrDev* ctr) {
  int nb = (int)std::min<long long>(120, (npts + 255) / 256);
  if (nb < 1) nb = 1;
  smc_eta_stats_apply_kernel<<<nb, 256, 0, c.s>>>(part, nb, eta, npts, law, ctr);
  SMC_LAUNCH_CHECK(c);
}

// whether the guard runs: min(eta) not > 0 (or a NaN), from the min/drift
// kernel's per-CTA partials (as its final reduction decides: any NaN partial
// makes the minimum NaN); every CTA takes the same decision
__device__ __forceinline__ bool eta_guard_active(const double* __restrict__ mpart, int mnp) {
  __shared__ int s_act;
  if (threadIdx.x < 32) {
    double a = INFINITY;
    bool nan_seen = false;
    for (int i = threadIdx.x; i < mnp; i += 32) {
      const double x = mpart[2 * i], y = mpart[2 * i + 1];
      if (x != x || y != y) nan_seen = true;
      a = fmin(a, x);
    }
    for (int d = 16; d > 0; d >>= 1) a = fmin(a, __shfl_xor_sync(0xffffffffu, a, d));
    nan_seen = __any_sync(0xffffffffu, nan_seen);
    if (threadIdx.x == 0) s_act = nan_seen || !(a > 0.0);
  }
  __syncthreads();
  return s_act != 0;
}

// guard, pass 1: per-CTA counts of the points outside the dead-band window
__global__ void smc_eta_guard_count_kernel(const double* __restrict__ mpart, int mnp,
                                           const double* __restrict__ eta, long long npts, EtaLaw law,
                                           double* __restrict__ part) {
  if (!eta_guard_active(mpart, mnp)) return;
  __shared__ double ws[8];
  double cnt = 0.0;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < npts;
       idx += (long long)gridDim.x * blockDim.x) {
    const double e = eta[idx];
    if (e < law.lo_eff || e > law.hi_eff) cnt += 1.0;
  }
  cnt = block_sum256(cnt, ws);
  if (threadIdx.x == 0) part[blockIdx.x] = cnt;
}

// guard, pass 2: every CTA sums the pass-1 counts (integers: exact in any
// order), CTA 0 adds them to the counters, and the window is applied when it
// is smooth or some point lies outside the dead band
__global__ void smc_eta_guard_apply_kernel(const double* __restrict__ mpart, int mnp,
                                           double* __restrict__ eta, long long npts, EtaLaw law,
                                           const double* __restrict__ part, int np,
                                           EtaCtrDev* __restrict__ ctr) {
  if (!eta_guard_active(mpart, mnp)) return;
  __shared__ double ws[8];
  __shared__ double s_c;
  if (threadIdx.x < 32) {
    double c = 0.0;
    for (int b = threadIdx.x; b < np; b += 32) c += part[b];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (threadIdx.x == 0) s_c = c;
  }
  __syncthreads();
  const double c = s_c;
  if (blockIdx.x == 0 && threadIdx.x == 0) ctr->n_clip_eta_proj += (long long)c;
  if (!(law.w > 0.0) && !(c > 0.0)) return;
  double band = 0.0;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < npts;
       idx += (long long)gridDim.x * blockDim.x)
    eta[idx] = eta_window_value(eta[idx], law, band);
  if (!(law.w > 0.0)) return;
  band = block_sum256(band, ws);
  if (threadIdx.x == 0 && band > 0.0)
    atomicAdd(reinterpret_cast<unsigned long long*>(&ctr->n_smooth_eta_proj),
              (unsigned long long)(long long)band);
}

void eta_guard(const Ctx& c, const double* mpart, double* eta, long long npts, const EtaLaw& law,
               EtaCtrDev* ctr, double* scratch) {
  int nb = (int)std::min<long long>(120, (npts + 255) / 256);
  if (nb < 1) nb = 1;
  smc_eta_guard_count_kernel<<<nb, 256, 0, c.s>>>(mpart, nb, eta, npts, law, scratch);
  SMC_LAUNCH_CHECK(c);
  smc_eta_guard_apply_kernel<<<nb, 256, 0, c.s>>>(mpart, nb, eta, npts, law, scratch, nb, ctr);
  SMC_LAUNCH_CHECK(c);
}

// ------------------------------------------------ BFBT block reuse decision
__global__ void smc_bfbt_decide_kernel(const double2* __restrict__ prof, double2* __restrict__ held,
                                       int N, int max_age, double rel, BfbtHold* __restrict__ h,
                                       cudaGraphConditionalHandle cond) {
  __shared__ double wmx[8], wmd[8];
  __shared__ int s_reuse;
  const int valid = h->valid, age = h->age;
  if (valid && age < max_age) {
    double mx = 0.0, md = 0.0;       // fmax drops NaN operands, as host_max does
    for (int q = threadIdx.x; q < N; q += blockDim.x) {
      const double hq = held[q].x;
      mx = fmax(mx, fabs(hq));
      md = fmax(md, fabs(prof[q].x - hq));
    }
    for (int o = 16; o > 0; o >>= 1) {
      mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      md = fmax(md, __shfl_xor_sync(0xffffffffu, md, o));
    }
    if ((threadIdx.x & 31) == 0) { wmx[threadIdx.x >> 5] = mx; wmd[threadIdx.x >> 5] = md; }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { mx = fmax(mx, wmx[q]); md = fmax(md, wmd[q]); }
      s_reuse = isfinite(md) && md <= rel * mx;
    }
  } else if (threadIdx.x == 0) {
    s_reuse = 0;
  }
  __syncthreads();
  const int reuse = s_reuse;
  if (!reuse)
    for (int q = threadIdx.x; q < N; q += blockDim.x) held[q] = prof[q];
  if (threadIdx.x == 0) {
    h->valid = 1;
    h->age = reuse ? age + 1 : 1;
    cudaGraphSetConditional(cond, reuse ? 0u : 1u);
  }
}

void bfbt_decide(const Ctx& c, const double2* prof, double2* held, int N, int max_age, double rel,
                 BfbtHold* h, cudaGraphConditionalHandle cond) {
  smc_bfbt_decide_kernel<<<1, 256, 0, c.s>>>(prof, held, N, max_age, rel, h, cond);
  SMC_LAUNCH_CHECK(c);
}

// harmonic mean over x of the (Nx, N) field: g_j = 1 / mean_i(1/eta[i][j])
// out_j = w_j / mean_i(1 / eta[i][j]); one CTA per column j: the reciprocals
// (FP64 divisions, the expensive part) in parallel, then the column sum by
// one thread in the order i = 0, 1, ..., in chunks of HP_CHUNK.  The sum
// order is that of a row-by-row reduction over axis 0 whatever the launch
// shape, and the FP64 divisions are spread over N SMs instead of one.
static constexpr int HP_CHUNK = 1024;
__global__ void smc_harm_profile_kernel(const double* __restrict__ eta, int Nx, int N,
                                        const double* __restrict__ wq, double2* __restrict__ out) {
  __shared__ double rcp[HP_CHUNK];
  const int j = blockIdx.x;
  double s = 0.0;
  for (int base = 0; base < Nx; base += HP_CHUNK) {
    const int cnt = min(HP_CHUNK, Nx - base);
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) rcp[i] = 1.0 / eta[(long long)(base + i) * N + j];
    __syncthreads();
    if (threadIdx.x == 0)
      for (int i = 0; i < cnt; ++i) s += rcp[i];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[j] = make_double2(wq[j] * (1.0 / (s / Nx)), 0.0);
}

void harm_profile_rhs(const Ctx& c, const double* eta, int Nx, int N, const double* wq,
                      double2* out) {
  smc_harm_profile_kernel<<<N, 128, 0, c.s>>>(eta, Nx, N, wq, out);
  SMC_LAUNCH_CHECK(c);
}

// real Chebyshev product matrix of a real coefficient vector a (row-major)
__global__ void smc_cheb_mult_real_kernel(const double* __restrict__ a, double* __restrict__ M, int N) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  int p = blockIdx.y;
  if (q >= N) return;
  double s = 0.0;
  if (p >= q) s += a[p - q];
  if (p + q < N) s += a[p + q];
  if (p > 0 && q >= p) s += a[q - p];
  M[(long long)p * N + q] = 0.5 * s;
}

void cheb_mult_real(const Ctx& c, const double* a, double* M, int N) {
  dim3 grd(ceil_div(N, 128), N);
  smc_cheb_mult_real_kernel<<<grd, 128, 0, c.s>>>(a, M, N);
  SMC_LAUNCH_CHECK(c);
}

// reduced operator blocks (row-major in, column-major LU layout out):
//   P_k = (D2 - k^2 I) M + 2 k^2 (Comm G_k),  rows N-2, N-1 = V[0], V[N-1]
// CommG = Comm G_k precomputed per k; DM = D2 M
__global__ void smc_reduced_blocks_kernel(const double* __restrict__ DM, const double* __restrict__ M,
                                          const double* __restrict__ CommG, const double* __restrict__ V,
                                          const double* __restrict__ kx, double* __restrict__ Pcm,
                                          int N) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  int p = blockIdx.y;
  int k = blockIdx.z;
  if (q >= N) return;
  long long NN = (long long)N * N;
  double v;
  if (p == N - 2) v = V[q];
  else if (p == N - 1) v = V[(long long)(N - 1) * N + q];
  else {
    double kk = kx[k] * kx[k];
    long long e = (long long)p * N + q;
    v = (DM[e] - kk * M[e]) + 2.0 * kk * CommG[k * NN + e];
  }
  Pcm[k * NN + (long long)q * N + p] = v;
}

void reduced_blocks(const Ctx& c, const double* DM, const double* M, const double* CommG,
                    const double* V, const double* kx, double* Pcm, int N, int Nk) {
  dim3 grd(ceil_div(N, 128), N, Nk);
  smc_reduced_blocks_kernel<<<grd, 128, 0, c.s>>>(DM, M, CommG, V, kx, Pcm, N);
  SMC_LAUNCH_CHECK(c);
}

// Helmholtz tau operators (column-major): D2 - (k^2 + lam) I, rows N-2 =
// (-1)^n (u(0)), N-1 = 1 (u(1))   (rbc_galerkin.py:162-168)
__global__ void smc_tau_ops_kernel(const double* __restrict__ D2, const double* __restrict__ kx,
                                   double lam, double* __restrict__ Acm, int N) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  int p = blockIdx.y;
  int k = blockIdx.z;
  if (q >= N) return;
  double v;
  if (p == N - 2) v = (q & 1) ? -1.0 : 1.0;
  else if (p == N - 1) v = 1.0;
  else v = D2[(long long)p * N + q] - ((p == q) ? (kx[k] * kx[k] + lam) : 0.0);
  Acm[(long long)k * N * N + (long long)q * N + p] = v;
}

void tau_ops(const Ctx& c, const double* D2, const double* kx, double lam, double* Acm, int N,
             int Nk) {
  dim3 grd(ceil_div(N, 128), N, Nk);
  smc_tau_ops_kernel<<<grd, 128, 0, c.s>>>(D2, kx, lam, Acm, N);
  SMC_LAUNCH_CHECK(c);
}

}  // namespace smc
