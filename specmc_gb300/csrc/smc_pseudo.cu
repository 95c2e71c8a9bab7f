// Pseudo-spectral evaluation of mult_eta (stokes/lagged_stokes.py:162-193).
//
// mult_eta(f)_i = sum_j M_{i-j} f_j + sgn sum_{m>=1} M_{i+m} f_m, i in [0, Nk),
// with M_d the exact truncated Chebyshev product by a_d = eta_c[d]
// (a_{-d} = conj(a_d)).  With F_j = f_j (j >= 0), F_{-m} = sgn f_m (m >= 1),
// this is the linear x-convolution (a * F)_i restricted to i in [0, Nk),
// each term an exact Chebyshev product truncated to N coefficients.  Both
// products are evaluated on a grid:
//   x: a DFT of length L >= 3 Nk - 2 (no alias of the support
//      [-2Nk+2, 2Nk-2] reaches the kept modes [0, Nk));
//   z: values at Mz = 2N - 1 CGL points, where the degree <= 2N - 2 product
//      is interpolated exactly; the first N Chebyshev coefficients of the
//      interpolant are the truncated product.
// The linear map is identical to the dense block form; only the arithmetic
// order differs (roundoff level).  Work per call ~ Nk Mz (N + 3L) complex
// MACs instead of ~1.5 Nk^2 N^2.
#include "smc_internal.cuh"
#include "smc_pseudo.cuh"
#include "smc_fft.cuh"

namespace smc {

// Fv[b][j][s] = sum_q Zf[s][q] f_b[j][q]   (Nk x Mz per field)
__global__ void __launch_bounds__(128) smc_ps_zfwd_kernel(PsJobs jobs, const double* __restrict__ Zf,
                                                          int Nk, int N, int Mz,
                                                          double2* __restrict__ Fv) {
  // CSPLIT lanes per output (FP64-pipe bound, as smc_zmat_kernel)
  const int sub = threadIdx.x & (CSPLIT - 1);
  const int s = blockIdx.x * (blockDim.x / CSPLIT) + threadIdx.x / CSPLIT;
  const int j = blockIdx.y, b = blockIdx.z;
  double sr = 0.0, si = 0.0;
  if (s < Mz) {
    const double2* f = jobs.f[b] + (long long)j * N;
    const double* z = Zf + (long long)s * N;
    for (int q = sub; q < N; q += CSPLIT) {
      double w = z[q];
      double2 v = f[q];
      sr += w * v.x;
      si += w * v.y;
    }
  }
  sr = split8_sum(sr);
  si = split8_sum(si);
  if (s < Mz && sub == 0) Fv[((long long)b * Nk + j) * Mz + s] = make_double2(sr, si);
}

// Per z-point s and field b: G(l) = sum_j F_j e^{2 pi i j l/L}, P = E G,
// H_i = (1/L) sum_l P(l) e^{-2 pi i i l/L}, i < Nk.
__global__ void smc_ps_x_kernel(const double2* __restrict__ Fv, const double* __restrict__ E,
                                PsJobs jobs, int Nk, int Mz, int L, const double2* __restrict__ tw,
                                double2* __restrict__ Hv) {
  extern __shared__ double2 sm[];
  double2* P = sm;          // L
  double2* W = sm + L;      // L/2 twiddles
  const int s = blockIdx.x, b = blockIdx.y, tid = threadIdx.x, nt = blockDim.x;
  const double sgn = jobs.sgn[b];
  const int logL = ilog2_pow2(L);
  for (int i = tid; i < (L >> 1); i += nt) W[i] = tw[i];
  for (int i = tid; i < L; i += nt) P[i] = make_double2(0.0, 0.0);
  __syncthreads();
  // G(l) = sum_j F_j e^{+i th} + sgn sum_{j>=1} F_j e^{-i th}: the modes at
  // +j and (the partner sign times) at L - j, then one inverse-direction FFT
  for (int j = tid; j < Nk; j += nt) {
    const double2 f = Fv[((long long)b * Nk + j) * Mz + s];
    P[j] = f;
    if (j > 0) P[L - j] = make_double2(sgn * f.x, sgn * f.y);
  }
  __syncthreads();
  cta_fft(P, L, logL, W, +1, tid, nt);
  for (int l = tid; l < L; l += nt) {
    const double e = E[(long long)l * Mz + s];
    P[l] = make_double2(e * P[l].x, e * P[l].y);
  }
  __syncthreads();
  // H_i = (1/L) sum_l P(l) e^{-i th}, i < Nk
  cta_fft(P, L, logL, W, -1, tid, nt);
  const double invL = 1.0 / L;
  for (int i = tid; i < Nk; i += nt)
    Hv[((long long)b * Nk + i) * Mz + s] = make_double2(P[i].x * invL, P[i].y * invL);
}

// out_b[i][p] = sum_s Zi[p][s] Hv[b][i][s]
__global__ void smc_ps_zinv_kernel(const double2* __restrict__ Hv, const double* __restrict__ Zi,
                                   PsJobs jobs, int Nk, int N, int Mz) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y, b = blockIdx.z;
  if (p >= N) return;
  const double2* h = Hv + ((long long)b * Nk + i) * Mz;
  const double* z = Zi + (long long)p * Mz;
  double sr = 0.0, si = 0.0;
  for (int s = 0; s < Mz; ++s) {
    double w = z[s];
    sr += w * h[s].x;
    si += w * h[s].y;
  }
  jobs.out[b][(long long)i * N + p] = make_double2(sr, si);
}

// E[l][s] = Re a_0(z_s) + 2 Re sum_{d>=1} a_d(z_s) e^{2 pi i d l/L}
__global__ void smc_ps_eta_grid_kernel(const double2* __restrict__ Av, int Nk, int Mz, int L,
                                       const double2* __restrict__ tw, double* __restrict__ E) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int l = blockIdx.y;
  if (s >= Mz) return;
  double acc = 0.0;
  int idx = 0;                           // d l mod L, stepped (l < L)
  for (int d = 1; d < Nk; ++d) {
    idx += l;
    if (idx >= L) idx -= L;
    double2 a = Av[(long long)d * Mz + s];
    double2 t = tw[idx];
    acc += a.x * t.x - a.y * t.y;
  }
  E[(long long)l * Mz + s] = Av[s].x + 2.0 * acc;
}

void ps_eta_grid(const Ctx& c, const PsPlan& pl, const double2* eta_c, double2* work, double* E) {
  PsJobs j{};
  j.f[0] = eta_c;
  dim3 g1(ceil_div(pl.Mz, 128 / CSPLIT), pl.Nk, 1);
  smc_ps_zfwd_kernel<<<g1, 128, 0, c.s>>>(j, pl.Zf, pl.Nk, pl.N, pl.Mz, work);
  SMC_LAUNCH_CHECK(c);
  dim3 g2(ceil_div(pl.Mz, 128), pl.L);
  smc_ps_eta_grid_kernel<<<g2, 128, 0, c.s>>>(work, pl.Nk, pl.Mz, pl.L, pl.tw, E);
  SMC_LAUNCH_CHECK(c);
}

void ps_mult_eta(const Ctx& c, const PsPlan& pl, const double* E, const PsJobs& jobs, int nb,
                 double2* Fv, double2* Hv) {
  dim3 g1(ceil_div(pl.Mz, 128 / CSPLIT), pl.Nk, nb);
  smc_ps_zfwd_kernel<<<g1, 128, 0, c.s>>>(jobs, pl.Zf, pl.Nk, pl.N, pl.Mz, Fv);
  SMC_LAUNCH_CHECK(c);
  dim3 g2(pl.Mz, nb);
  size_t sm = (size_t)(pl.L + pl.L / 2) * sizeof(double2);
  allow_max_smem((const void*)smc_ps_x_kernel);
  smc_ps_x_kernel<<<g2, 128, sm, c.s>>>(Fv, E, jobs, pl.Nk, pl.Mz, pl.L, pl.tw, Hv);
  SMC_LAUNCH_CHECK(c);
  dim3 g3(ceil_div(pl.N, 128), pl.Nk, nb);
  smc_ps_zinv_kernel<<<g3, 128, 0, c.s>>>(Hv, pl.Zi, jobs, pl.Nk, pl.N, pl.Mz);
  SMC_LAUNCH_CHECK(c);
}

}  // namespace smc
