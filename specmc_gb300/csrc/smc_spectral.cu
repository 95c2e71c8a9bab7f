// Spectral transforms, pointwise grid kernels, vector kernels and reductions
// of the FP64 (plain) time step.
//
// The Fourier x Chebyshev transforms of SpecMC (specmc/core/rbc_galerkin.py:
// 322-339) are separable: a real N x N matrix along z (V, V^{-1}, D, D^2,
// G_k) and a real DFT along x.  At the grid sizes of this path (Nx <= 128,
// Nz <= 96) both are short dense contractions, so they are written as
// direct sums with precomputed twiddles instead of FFTs; the results agree
// with numpy's pocketfft to roundoff.
#include "smc_internal.cuh"
#include "smc_tc.cuh"

namespace smc {

struct ZJobs4 { ZJob j[4]; };
struct SynthJobs4 { SynthJob j[4]; };
struct AnaJobs4 { AnaJob j[4]; };

// ------------------------------------------------------------ z contraction
// GB300's FP64 pipe issues a warp-wide FMA over many cycles, so a
// contraction is bound by how many SM sub-partitions carry FP64 work: each
// output is summed by CSPLIT consecutive lanes (lane s takes m = s, s + 8, ...)
// and combined pairwise in a fixed order (split8_sum), which puts 8x more
// warps on the GPU than one thread per output and cuts each lane's chain of
// dependent FP64 FMAs to N / 8.
static constexpr int ZOUT = 16;          // outputs per 128-thread CTA

__global__ void __launch_bounds__(CSPLIT * ZOUT) smc_zmat_kernel(ZJobs4 jobs, int Nk, int N,
                                                                 const double* __restrict__ kx) {
  const ZJob& jb = jobs.j[blockIdx.z];
  const int sub = threadIdx.x & (CSPLIT - 1);
  const int n = blockIdx.x * ZOUT + threadIdx.x / CSPLIT;
  const int k = blockIdx.y;
  const bool act = n < N && k < Nk;
  const bool tau = act && jb.zero_tau && n >= N - 2;
  double sr = 0.0, si = 0.0;
  if (act && !tau) {
    const double* Zr = jb.Z + (long long)k * jb.zstride + (long long)n * N;
    const double2* xr = jb.X + (long long)k * N;
    if (jb.x_real) {
      for (int m = sub; m < N; m += CSPLIT) sr += Zr[m] * xr[m].x;
    } else {
      for (int m = sub; m < N; m += CSPLIT) {
        double z = Zr[m];
        double2 x = xr[m];
        sr += z * x.x;
        si += z * x.y;
      }
    }
  }
  sr = split8_sum(sr);
  si = split8_sum(si);
  if (!act || sub != 0) return;
  double2* yp = jb.Y + (long long)k * N + n;
  if (tau) {
    if (!jb.accumulate) *yp = make_double2(0.0, 0.0);
    return;
  }
  double2 f = kfactor_eval(jb.f, kx ? kx[k] : 0.0);
  double2 r = make_double2(f.x * sr - f.y * si, f.x * si + f.y * sr);
  if (jb.accumulate) r = cadd(*yp, r);
  *yp = r;
}

void zmat_apply(const Ctx& c, const ZJob* jobs, int njobs, int Nk, int N, const double* kx) {
  if (njobs < 1 || njobs > 4) throw std::runtime_error("zmat_apply: 1..4 jobs");
  // shared operators of up to 128 columns go to the tensor cores when the
  // handle has them enabled (same result to FP64 roundoff, smc_tc.cu)
  if (c.tc && tc_zmat_apply(c, *c.tc, jobs, njobs, Nk, N, kx)) return;
  ZJobs4 js;
  for (int i = 0; i < njobs; ++i) js.j[i] = jobs[i];
  dim3 blk(CSPLIT * ZOUT), grd(ceil_div(N, ZOUT), Nk, njobs);
  smc_zmat_kernel<<<grd, blk, 0, c.s>>>(js, Nk, N, kx);
  SMC_LAUNCH_CHECK(c);
}

// ------------------------------------------------------------ x synthesis
// g[i][j] = Re X[0][j] + sum_{k>=1} w_k Re(X[k][j] e^{2 pi i k i/Ng}),
// w_k = 2, except the Nyquist mode 2k == Ng (weight 1, Re only) -- the
// Hermitian reconstruction numpy.fft.irfft performs.
__global__ void __launch_bounds__(CSPLIT * ZOUT) smc_synth_x_kernel(SynthJobs4 jobs, int Nk, int N, int Ng,
                                                                    const double2* __restrict__ tw) {
  // CSPLIT lanes per output (as smc_zmat_kernel): lane sub takes the modes
  // k = 1 + sub, 1 + sub + 8, ...; the mode-0 term is added to the lane sum
  const SynthJob& jb = jobs.j[blockIdx.z];
  const int sub = threadIdx.x & (CSPLIT - 1);
  const int j = blockIdx.x * ZOUT + threadIdx.x / CSPLIT;
  const int i = blockIdx.y;
  const bool act = j < N && i < Ng;
  double acc = 0.0;
  if (act) {
    int idx = (int)(((long long)(1 + sub) * i) % Ng);   // k i mod Ng, stepped by 8 i
    const int step = (int)(((long long)CSPLIT * i) % Ng);
    for (int k = 1 + sub; k < Nk; k += CSPLIT) {
      double2 x = jb.X[(long long)k * N + j];
      double2 t = tw[idx];
      idx += step;
      if (idx >= Ng) idx -= Ng;
      double v = x.x * t.x - x.y * t.y;
      acc += (2 * k == Ng) ? v : 2.0 * v;
    }
  }
  acc = split8_sum(acc);
  if (act && sub == 0) jb.g[(long long)i * N + j] = jb.X[j].x + acc;
}

void synth_x(const Ctx& c, const SynthJob* jobs, int njobs, int Nk, int N, int Ng,
             const double2* tw) {
  if (njobs < 1 || njobs > 4) throw std::runtime_error("synth_x: 1..4 jobs");
  SynthJobs4 js;
  for (int q = 0; q < njobs; ++q) js.j[q] = jobs[q];
  dim3 blk(CSPLIT * ZOUT), grd(ceil_div(N, ZOUT), Ng, njobs);
  smc_synth_x_kernel<<<grd, blk, 0, c.s>>>(js, Nk, N, Ng, tw);
  SMC_LAUNCH_CHECK(c);
}

// ------------------------------------------------------------- x analysis
__global__ void __launch_bounds__(CSPLIT * ZOUT) smc_analysis_x_kernel(AnaJobs4 jobs, int Nk, int N, int Ng,
                                                                       const double2* __restrict__ tw,
                                                                       double scale) {
  const AnaJob& jb = jobs.j[blockIdx.z];
  const int sub = threadIdx.x & (CSPLIT - 1);
  const int j = blockIdx.x * ZOUT + threadIdx.x / CSPLIT;
  const int k = blockIdx.y;
  const bool act = j < N && k < Nk;
  double sr = 0.0, si = 0.0;
  if (act) {
    // lane sub takes i = sub, sub + 8, ...: twiddle index k i mod Ng, stepped
    int idx = (int)(((long long)k * sub) % Ng);
    const int step = (int)(((long long)k * CSPLIT) % Ng);
    for (int i = sub; i < Ng; i += CSPLIT) {
      double g = jb.g[(long long)i * N + j];
      double2 t = tw[idx];
      idx += step;
      if (idx >= Ng) idx -= Ng;
      sr += g * t.x;
      si -= g * t.y;
    }
  }
  sr = split8_sum(sr);
  si = split8_sum(si);
  if (act && sub == 0) jb.A[(long long)k * N + j] = make_double2(sr * scale, si * scale);
}

void analysis_x(const Ctx& c, const AnaJob* jobs, int njobs, int Nk, int N, int Ng,
                const double2* tw, double scale) {
  if (njobs < 1 || njobs > 4) throw std::runtime_error("analysis_x: 1..4 jobs");
  AnaJobs4 js;
  for (int i = 0; i < njobs; ++i) js.j[i] = jobs[i];
  dim3 blk(CSPLIT * ZOUT), grd(ceil_div(N, ZOUT), Nk, njobs);
  smc_analysis_x_kernel<<<grd, blk, 0, c.s>>>(js, Nk, N, Ng, tw, scale);
  SMC_LAUNCH_CHECK(c);
}

// ------------------------------------------------------- pointwise on grids
// N = -(ux thx + uz thz) + uz [+ H]   (rbc_galerkin.py:415-418)
__global__ void smc_explicit_nl_kernel(const double* ux, const double* uz, const double* thx,
                                       const double* thz, double H, double* out, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v = -(ux[i] * thx[i] + uz[i] * thz[i]) + uz[i];
  if (H != 0.0) v = v + H;
  out[i] = v;
}

void grid_explicit_nonlinear(const Ctx& c, const double* ux, const double* uz,
                             const double* thx, const double* thz, double H, double* out,
                             long long npts) {
  smc_explicit_nl_kernel<<<ceil_div(npts, 256), 256, 0, c.s>>>(ux, uz, thx, thz, H, out, npts);
  SMC_LAUNCH_CHECK(c);
}

// -(ux vx + uz vz)   (implicit_theta.py:300-304)
__global__ void smc_advect_prod_kernel(const double* ux, const double* uz, const double* vx,
                                       const double* vz, double* out, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = -(ux[i] * vx[i] + uz[i] * vz[i]);
}

void grid_advect_product(const Ctx& c, const double* ux, const double* uz, const double* vx,
                         const double* vz, double* out, long long npts) {
  smc_advect_prod_kernel<<<ceil_div(npts, 256), 256, 0, c.s>>>(ux, uz, vx, vz, out, npts);
  SMC_LAUNCH_CHECK(c);
}

// Phi = 2 [eta] (gxx^2 + gzz^2 + 2 gxz^2 - gtr^2/3)  (physics/dissipation.py:352-362)
__global__ void smc_phi_kernel(const double* gxx, const double* gzz, const double* gxz,
                               const double* gtr, const double* eta_pad, double coef,
                               double* out, long long n, int accumulate) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double sq = gxx[i] * gxx[i] + gzz[i] * gzz[i] + 2.0 * gxz[i] * gxz[i];
  double tr = gtr ? gtr[i] : 0.0;
  double dev = sq - (1.0 / 3.0) * tr * tr;
  double phi = eta_pad ? 2.0 * eta_pad[i] * dev : 2.0 * dev;
  double v = coef * phi;
  out[i] = accumulate ? out[i] + v : v;
}

void grid_phi(const Ctx& c, const double* gxx, const double* gzz, const double* gxz,
              const double* gtr, const double* eta_pad, double coef, double* out_accum,
              long long npts, int accumulate) {
  smc_phi_kernel<<<ceil_div(npts, 256), 256, 0, c.s>>>(gxx, gzz, gxz, gtr, eta_pad, coef,
                                                       out_accum, npts, accumulate);
  SMC_LAUNCH_CHECK(c);
}

// ----------------------------------------------------------------- reductions
static constexpr int RED_BLOCKS = 120;

__device__ __forceinline__ double block_reduce_max(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : -INFINITY;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  return v;
}

__device__ __forceinline__ double block_reduce_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  return v;
}

// NaN-propagating max of |x| (numpy's .max() returns nan when any entry is nan)
__device__ __forceinline__ double nanmax_abs(double m, double x) {
  double a = fabs(x);
  if (a != a || m != m) return NAN;
  return a > m ? a : m;
}

__global__ void smc_maxabs2_kernel(const double* a, const double* b, long long n, double* part) {
  __shared__ double sh[32];
  double m = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    m = nanmax_abs(m, a[i]);
    if (b) m = nanmax_abs(m, b[i]);
  }
  bool nan_seen = (m != m);
  double r = block_reduce_max(nan_seen ? INFINITY : m, sh);
  int any_nan = __syncthreads_or(nan_seen);
  if (threadIdx.x == 0) part[blockIdx.x] = any_nan ? NAN : r;
}

__global__ void smc_max_partials_kernel(const double* part, int np, double* dst) {
  __shared__ double sh[32];
  double m = 0.0;
  bool nan_seen = false;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    double v = part[i];
    if (v != v) nan_seen = true; else m = fmax(m, v);
  }
  double r = block_reduce_max(m, sh);
  int any_nan = __syncthreads_or(nan_seen);
  if (threadIdx.x == 0) dst[0] = any_nan ? NAN : r;
}

void reduce_maxabs2(const Ctx& c, const double* a, const double* b, long long n, double* dst,
                    double* scratch) {
  int nb = (int)std::min<long long>(RED_BLOCKS, (n + 255) / 256);
  if (nb < 1) nb = 1;
  smc_maxabs2_kernel<<<nb, 256, 0, c.s>>>(a, b, n, scratch);
  SMC_LAUNCH_CHECK(c);
  smc_max_partials_kernel<<<1, 256, 0, c.s>>>(scratch, nb, dst);
  SMC_LAUNCH_CHECK(c);
}

__global__ void smc_norm2_kernel(const double2* x, long long n, double* part) {
  __shared__ double sh[32];
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double2 v = x[i];
    s += v.x * v.x + v.y * v.y;
  }
  double r = block_reduce_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = r;
}

__global__ void smc_sum_partials_sqrt_kernel(const double* part, int np, double* dst) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
  double r = block_reduce_sum(s, sh);
  if (threadIdx.x == 0) dst[0] = sqrt(r);
}

void vec_norm2(const Ctx& c, const double2* x, long long n, double* dst, double* scratch) {
  int nb = (int)std::min<long long>(RED_BLOCKS, (n + 255) / 256);
  if (nb < 1) nb = 1;
  smc_norm2_kernel<<<nb, 256, 0, c.s>>>(x, n, scratch);
  SMC_LAUNCH_CHECK(c);
  smc_sum_partials_sqrt_kernel<<<1, 256, 0, c.s>>>(scratch, nb, dst);
  SMC_LAUNCH_CHECK(c);
}

// memo test: {all bytes equal, max|X - cX|, max|cX|}
__global__ void smc_memo_kernel(const double2* th, const double2* cth, const double2* X,
                                const double2* cX, long long n, double* part) {
  __shared__ double sh[32];
  double neq = 0.0, md = 0.0, mc = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double2 a = th[i], b = cth[i];
    if (__double_as_longlong(a.x) != __double_as_longlong(b.x) ||
        __double_as_longlong(a.y) != __double_as_longlong(b.y))
      neq = 1.0;
    double2 d = csub(X[i], cX[i]);
    md = nanmax_abs(md, hypot(d.x, d.y));
    mc = nanmax_abs(mc, hypot(cX[i].x, cX[i].y));
  }
  double r0 = block_reduce_max(neq, sh);
  double r1 = block_reduce_max(md != md ? INFINITY : md, sh);
  double r2 = block_reduce_max(mc != mc ? INFINITY : mc, sh);
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x + 0] = r0;
    part[3 * blockIdx.x + 1] = r1;
    part[3 * blockIdx.x + 2] = r2;
  }
}

// one warp: maxima over the per-CTA partials
__global__ void smc_memo_final_kernel(const double* part, int np, double* dst) {
  const int lane = threadIdx.x & 31;
  if (threadIdx.x >= 32) return;
  double a = 0.0, b = 0.0, cc = 0.0;
  for (int i = lane; i < np; i += 32) {
    a = fmax(a, part[3 * i]);
    b = fmax(b, part[3 * i + 1]);
    cc = fmax(cc, part[3 * i + 2]);
  }
  for (int d = 16; d > 0; d >>= 1) {
    a = fmax(a, __shfl_xor_sync(0xffffffffu, a, d));
    b = fmax(b, __shfl_xor_sync(0xffffffffu, b, d));
    cc = fmax(cc, __shfl_xor_sync(0xffffffffu, cc, d));
  }
  if (lane == 0) {
    dst[0] = (a == 0.0) ? 1.0 : 0.0;
    dst[1] = b;
    dst[2] = cc;
  }
}

void memo_compare(const Ctx& c, const double2* that, const double2* cthat, const double2* X,
                  const double2* cX, long long n, double* dst, double* scratch) {
  int nb = (int)std::min<long long>(RED_BLOCKS, (n + 255) / 256);
  if (nb < 1) nb = 1;
  smc_memo_kernel<<<nb, 256, 0, c.s>>>(that, cthat, X, cX, n, scratch);
  SMC_LAUNCH_CHECK(c);
  smc_memo_final_kernel<<<1, 32, 0, c.s>>>(scratch, nb, dst);
  SMC_LAUNCH_CHECK(c);
}

// ------------------------------------------------------------ vector kernels
__global__ void smc_axpby_kernel(double2* y, double2 a, const double2* x, double2 b, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 r = cmul(a, x[i]);
  if (b.x != 0.0 || b.y != 0.0) r = cadd(r, cmul(b, y[i]));
  y[i] = r;
}

void vec_axpby(const Ctx& c, double2* y, double2 a, const double2* x, double2 b, long long n) {
  smc_axpby_kernel<<<ceil_div(n, 256), 256, 0, c.s>>>(y, a, x, b, n);
  SMC_LAUNCH_CHECK(c);
}

void vec_copy(const Ctx& c, double2* y, const double2* x, long long n) {
  SMC_CUDA(cudaMemcpyAsync(y, x, n * sizeof(double2), cudaMemcpyDeviceToDevice, c.s));
}

void vec_zero(const Ctx& c, void* p, long long bytes) {
  SMC_CUDA(cudaMemsetAsync(p, 0, bytes, c.s));
}

__global__ void smc_scaled_modes_kernel(const double2* in, double2* out, int Nk, int N,
                                        KFactor f, const double* kx, int zero_tau, int zero_k0) {
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (n >= N || k >= Nk) return;
  long long i = (long long)k * N + n;
  double kk = kx[k];
  if ((zero_tau && n >= N - 2) || (zero_k0 && kk == 0.0)) {
    out[i] = make_double2(0.0, 0.0);
    return;
  }
  out[i] = cmul(kfactor_eval(f, kk), in[i]);
}

void vec_scaled_modes(const Ctx& c, const double2* in, double2* out, int Nk, int N, KFactor f,
                      const double* kx, int zero_tau, int zero_k0) {
  dim3 grd(ceil_div(N, 128), Nk);
  smc_scaled_modes_kernel<<<grd, 128, 0, c.s>>>(in, out, Nk, N, f, kx, zero_tau, zero_k0);
  SMC_LAUNCH_CHECK(c);
}

}  // namespace smc
