// Route kernels of the FP64 time step: the operator epilogues of the implicit
// temperature matvec and the matrix-free Schur matvec, the right-hand sides,
// the Arnoldi step of FGMRES and the diagnostics reduction.
#include "smc_internal.cuh"
#include "smc_route.cuh"

namespace smc {

// out = a0 v - (D2 v - k^2 v) - Vi A ; rows N-2, N-1 = v(z=0), v(z=1)
// (implicit_theta.py:354-383)
__global__ void smc_theta_combine_kernel(const double2* __restrict__ v, const double2* __restrict__ A,
                                         const double* __restrict__ D2, const double* __restrict__ Vi,
                                         const double* __restrict__ V, const double* __restrict__ kx,
                                         double a0, double2* __restrict__ out, int Nk, int N) {
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (n >= N || k >= Nk) return;
  const double2* vk = v + (long long)k * N;
  double2 r;
  if (n >= N - 2) {
    const double* Vr = V + (n == N - 2 ? 0 : (long long)(N - 1) * N);
    double sr = 0, si = 0;
    for (int m = 0; m < N; ++m) { sr += vk[m].x * Vr[m]; si += vk[m].y * Vr[m]; }
    r = make_double2(sr, si);
  } else {
    const double* Dr = D2 + (long long)n * N;
    const double* Vir = Vi + (long long)n * N;
    const double2* Ak = A + (long long)k * N;
    double lr = 0, li = 0, ar = 0, ai = 0;
    for (int m = 0; m < N; ++m) {
      lr += Dr[m] * vk[m].x; li += Dr[m] * vk[m].y;
      ar += Vir[m] * Ak[m].x; ai += Vir[m] * Ak[m].y;
    }
    double k2 = kx[k] * kx[k];
    double2 vn = vk[n];
    lr -= k2 * vn.x; li -= k2 * vn.y;
    r = make_double2((a0 * vn.x - lr) - ar, (a0 * vn.y - li) - ai);
  }
  out[(long long)k * N + n] = r;
}

void theta_combine(const Ctx& c, const double2* v, const double2* A, const double* D2,
                   const double* Vi, const double* V, const double* kx, double a0, double2* out,
                   int Nk, int N) {
  dim3 grd(ceil_div(N, 128), Nk);
  smc_theta_combine_kernel<<<grd, 128, 0, c.s>>>(v, A, D2, Vi, V, kx, a0, out, Nk, N);
  SMC_LAUNCH_CHECK(c);
}

// out = (D2 t1 - k^2 t1) + D2 t2 + 2k^2 t3 - 4k D t4 ; tau rows v(0), v(1)
// (stokes/lagged_stokes.py:215-220)
__global__ void smc_schur_combine_kernel(const double2* __restrict__ t1, const double2* __restrict__ t2,
                                         const double2* __restrict__ t3, const double2* __restrict__ t4,
                                         const double2* __restrict__ v, const double* __restrict__ D,
                                         const double* __restrict__ D2, const double* __restrict__ V,
                                         const double* __restrict__ kx, double2* __restrict__ out,
                                         int Nk, int N) {
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (n >= N || k >= Nk) return;
  long long o = (long long)k * N;
  double2 r;
  if (n >= N - 2) {
    const double* Vr = V + (n == N - 2 ? 0 : (long long)(N - 1) * N);
    double sr = 0, si = 0;
    for (int m = 0; m < N; ++m) { sr += v[o + m].x * Vr[m]; si += v[o + m].y * Vr[m]; }
    r = make_double2(sr, si);
  } else {
    const double* D2r = D2 + (long long)n * N;
    const double* Dr = D + (long long)n * N;
    double ar = 0, ai = 0, br = 0, bi = 0, dr = 0, di = 0;
    for (int m = 0; m < N; ++m) {
      ar += D2r[m] * t1[o + m].x; ai += D2r[m] * t1[o + m].y;
      br += D2r[m] * t2[o + m].x; bi += D2r[m] * t2[o + m].y;
      dr += Dr[m] * t4[o + m].x; di += Dr[m] * t4[o + m].y;
    }
    double kk = kx[k], k2 = kk * kk;
    double2 a1 = t1[o + n], a3 = t3[o + n];
    double xr = ar - k2 * a1.x, xi = ai - k2 * a1.y;
    xr = xr + br; xi = xi + bi;
    xr = xr + 2.0 * k2 * a3.x; xi = xi + 2.0 * k2 * a3.y;
    xr = xr - 4.0 * kk * dr; xi = xi - 4.0 * kk * di;
    r = make_double2(xr, xi);
  }
  out[o + n] = r;
}

void schur_combine(const Ctx& c, const double2* t1, const double2* t2, const double2* t3,
                   const double2* t4, const double2* v, const double* D, const double* D2,
                   const double* V, const double* kx, double2* out, int Nk, int N) {
  dim3 grd(ceil_div(N, 128), Nk);
  smc_schur_combine_kernel<<<grd, 128, 0, c.s>>>(t1, t2, t3, t4, v, D, D2, V, kx, out, Nk, N);
  SMC_LAUNCH_CHECK(c);
}

// rhs = that/dt + Nc   (rbc_galerkin.py:431)
__global__ void smc_const_rhs_kernel(const double2* th, const double2* Nc, double dt, double2* out,
                                     long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = make_double2(th[i].x / dt + Nc[i].x, th[i].y / dt + Nc[i].y);
}

void const_rhs(const Ctx& c, const double2* th, const double2* Nc, double dt, double2* out,
               long long n) {
  smc_const_rhs_kernel<<<ceil_div(n, 256), 256, 0, c.s>>>(th, Nc, dt, out, n);
  SMC_LAUNCH_CHECK(c);
}

// b = b0 th - b1 prev + (-i k psi) ; tau columns 0 ; b[0][0] += H ;
// rows < N-2 += phi  (implicit_theta.py:385-449)
__global__ void smc_theta_rhs_kernel(const double2* __restrict__ th, const double2* __restrict__ prev,
                                     const double2* __restrict__ psi, const double2* __restrict__ phi,
                                     const double* __restrict__ kx, double b0, double b1, double H,
                                     double2* __restrict__ b, int Nk, int N) {
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (n >= N || k >= Nk) return;
  long long i = (long long)k * N + n;
  if (n >= N - 2) { b[i] = make_double2(0.0, 0.0); return; }
  double2 v = make_double2(b0 * th[i].x, b0 * th[i].y);
  if (b1 != 0.0) v = make_double2(v.x - b1 * prev[i].x, v.y - b1 * prev[i].y);
  double kk = kx[k];
  double2 p = psi[i];
  // (-i k) * psi = (k psi.y, -k psi.x)
  v = make_double2(v.x + kk * p.y, v.y - kk * p.x);
  if (H != 0.0 && i == 0) v.x += H;
  if (phi) v = cadd(v, phi[i]);
  b[i] = v;
}

void theta_rhs(const Ctx& c, const double2* th, const double2* prev, const double2* psi,
               const double2* phi, const double* kx, double b0, double b1, double H, double2* b,
               int Nk, int N) {
  dim3 grd(ceil_div(N, 128), Nk);
  smc_theta_rhs_kernel<<<grd, 128, 0, c.s>>>(th, prev, psi, phi, kx, b0, b1, H, b, Nk, N);
  SMC_LAUNCH_CHECK(c);
}

// 2 psi - psi_prev   (implicit_theta.py:283-285)
__global__ void smc_extrap_kernel(const double2* a, const double2* b, double2* out, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = make_double2(2.0 * a[i].x - b[i].x, 2.0 * a[i].y - b[i].y);
}

void extrapolate(const Ctx& c, const double2* a, const double2* b, double2* out, long long n) {
  smc_extrap_kernel<<<ceil_div(n, 256), 256, 0, c.s>>>(a, b, out, n);
  SMC_LAUNCH_CHECK(c);
}

// out = in / h (real h)
__global__ void smc_div_kernel(const double2* in, double h, double2* out, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = make_double2(in[i].x / h, in[i].y / h);
}

void vec_div(const Ctx& c, const double2* in, double h, double2* out, long long n) {
  smc_div_kernel<<<ceil_div(n, 256), 256, 0, c.s>>>(in, h, out, n);
  SMC_LAUNCH_CHECK(c);
}

// Modified Gram-Schmidt of w against V_0..V_j, then ||w|| (krylov_fgmres.py:
// 139-144).  One CTA: the j+1 projections are sequential by construction.
__global__ void __launch_bounds__(1024) smc_mgs_kernel(const double2* __restrict__ Vb, int j,
                                                      long long n, double2* __restrict__ w,
                                                      double2* __restrict__ hout) {
  __shared__ double shr[32], shi[32];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5;
  for (int i = 0; i <= j; ++i) {
    const double2* Vi = Vb + (long long)i * n;
    double sr = 0.0, si = 0.0;
    for (long long t = tid; t < n; t += nt) {
      double2 a = Vi[t], b = w[t];          // conj(a) * b
      sr += a.x * b.x + a.y * b.y;
      si += a.x * b.y - a.y * b.x;
    }
    for (int o = 16; o > 0; o >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
      si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if (lane == 0) { shr[wid] = sr; shi[wid] = si; }
    __syncthreads();
    if (wid == 0) {
      sr = (lane < (nt >> 5)) ? shr[lane] : 0.0;
      si = (lane < (nt >> 5)) ? shi[lane] : 0.0;
      for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
        si += __shfl_xor_sync(0xffffffffu, si, o);
      }
      if (lane == 0) { shr[0] = sr; shi[0] = si; }
    }
    __syncthreads();
    const double2 h = make_double2(shr[0], shi[0]);
    __syncthreads();
    for (long long t = tid; t < n; t += nt) w[t] = csub(w[t], cmul(h, Vi[t]));
    if (tid == 0) hout[i] = h;
    __syncthreads();
  }
  double s = 0.0;
  for (long long t = tid; t < n; t += nt) s += w[t].x * w[t].x + w[t].y * w[t].y;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) shr[wid] = s;
  __syncthreads();
  if (tid == 0) {
    double a = 0.0;
    for (int q = 0; q < (nt >> 5); ++q) a += shr[q];
    hout[j + 1] = make_double2(sqrt(a), 0.0);
  }
}

void mgs(const Ctx& c, const double2* V, int j, long long n, double2* w, double2* hout) {
  smc_mgs_kernel<<<1, 1024, 0, c.s>>>(V, j, n, w, hout);
  SMC_LAUNCH_CHECK(c);
}

// x += sum_{j<k} y_j Z_j
__global__ void smc_krylov_update_kernel(double2* __restrict__ x, const double2* __restrict__ Z,
                                         const double2* __restrict__ y, int k, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 s = make_double2(0.0, 0.0);
  for (int j = 0; j < k; ++j) s = cadd(s, cmul(y[j], Z[(long long)j * n + i]));
  x[i] = cadd(x[i], s);
}

void krylov_update(const Ctx& c, double2* x, const double2* Z, const double2* y, int k,
                   long long n) {
  smc_krylov_update_kernel<<<ceil_div(n, 256), 256, 0, c.s>>>(x, Z, y, k, n);
  SMC_LAUNCH_CHECK(c);
}

// RBC.diagnostics (rbc_galerkin.py:439-453) from the grids ux, uz, th (Nx, N)
// and the k = 0 row of that.  out = {Nu_top, Nu_bot, Nu_energy, urms, umax, amp}
// CTA g takes DIAG_COLS columns of the grids (32 row slices per column,
// summed in slice order) and the same rows of D theta_0 (one warp per row),
// and writes its weighted sums and maxima; the last CTA to finish (a ticket,
// reset for the next launch) adds the CTAs' partials in CTA order.  The
// arithmetic is spread over ceil(N / 8) SMs: FP64 on GB300 runs at about two
// lanes per clock per SM, so one CTA spent 33 us on it at 64x96.
constexpr int DIAG_COLS = 8, DIAG_SLICES = 32, DIAG_THREADS = DIAG_COLS * DIAG_SLICES;
__global__ void __launch_bounds__(DIAG_THREADS) smc_diag_kernel(
    const double* __restrict__ ux, const double* __restrict__ uz, const double* __restrict__ th,
    const double2* __restrict__ that0, const double* __restrict__ D, const double* __restrict__ V,
    const double* __restrict__ wq, int Nx, int N, double* __restrict__ part,
    unsigned int* __restrict__ ticket, double* __restrict__ out) {
  __shared__ double ps[4][DIAG_SLICES][DIAG_COLS];
  __shared__ double fl[2][DIAG_COLS];
  __shared__ int s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c0 = blockIdx.x * DIAG_COLS;
  {
    const int jc = threadIdx.x % DIAG_COLS, sl = threadIdx.x / DIAG_COLS, j = c0 + jc;
    double a = 0, b = 0, m = 0, t = 0;
    if (j < N)
      for (int i = sl; i < Nx; i += DIAG_SLICES) {
        const long long e = (long long)i * N + j;
        const double x = ux[e], z = uz[e], h = th[e];
        a += x * x + z * z;
        b += z * h;
        m = fmax(m, fmax(fabs(x), fabs(z)));
        t = fmax(t, fabs(h));
      }
    ps[0][sl][jc] = a;
    ps[1][sl][jc] = b;
    ps[2][sl][jc] = m;
    ps[3][sl][jc] = t;
  }
  {
    // (D theta_0)[r] for this CTA's rows r = c0 + warp, and its boundary fluxes
    const int r = c0 + warp;
    double d = 0;
    if (r < N)
      for (int q = lane; q < N; q += 32) d += D[(long long)r * N + q] * that0[q].x;
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    if (lane == 0) {
      fl[0][warp] = r < N ? V[(long long)(N - 1) * N + r] * d : 0.0;
      fl[1][warp] = r < N ? V[r] * d : 0.0;
    }
  }
  __syncthreads();
  // one thread per column sums its slices (dependent FP64 chains stay short);
  // thread 0 then forms the quadrature-weighted sums in column order
  __shared__ double cs[4][DIAG_COLS];
  if (threadIdx.x < DIAG_COLS) {
    const int jc = threadIdx.x;
    double a = 0, b = 0, mm = 0, tt = 0;
    if (c0 + jc < N) {
      for (int sl = 0; sl < DIAG_SLICES; ++sl) {
        a += ps[0][sl][jc];
        b += ps[1][sl][jc];
        mm = fmax(mm, ps[2][sl][jc]);
        tt = fmax(tt, ps[3][sl][jc]);
      }
      cs[0][jc] = a / Nx;
      cs[1][jc] = b / Nx;
    }
    cs[2][jc] = mm;
    cs[3][jc] = tt;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double v1 = 0, v2 = 0, m = 0, t = 0, ntop = 0, nbot = 0;
    for (int jc = 0; jc < DIAG_COLS && c0 + jc < N; ++jc) {
      v1 += wq[c0 + jc] * cs[0][jc];
      v2 += wq[c0 + jc] * cs[1][jc];
      m = fmax(m, cs[2][jc]);
      t = fmax(t, cs[3][jc]);
      ntop += fl[0][jc];
      nbot += fl[1][jc];
    }
    double* p = part + 6LL * blockIdx.x;
    p[0] = v1; p[1] = v2; p[2] = m; p[3] = t; p[4] = ntop; p[5] = nbot;
    __threadfence();
    s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last || threadIdx.x != 0) return;
  __threadfence();
  double v1 = 0, v2 = 0, m = 0, t = 0, ntop = 0, nbot = 0;
  for (int g = 0; g < (int)gridDim.x; ++g) {
    const volatile double* p = part + 6LL * g;
    v1 += p[0]; v2 += p[1]; m = fmax(m, p[2]); t = fmax(t, p[3]); ntop += p[4]; nbot += p[5];
  }
  out[0] = 1.0 - ntop;
  out[1] = 1.0 - nbot;
  out[2] = 1.0 + v2;
  out[3] = sqrt(fmax(v1, 0.0));
  out[4] = m;
  out[5] = t;
  *ticket = 0u;
}

void diagnostics_reduce(const Ctx& c, const double* ux, const double* uz, const double* th,
                        const double2* that0, const double* D, const double* V, const double* wq,
                        int Nx, int N, double* out, double* scratch, unsigned int* ticket) {
  const int G = (N + DIAG_COLS - 1) / DIAG_COLS;
  smc_diag_kernel<<<G, DIAG_THREADS, 0, c.s>>>(ux, uz, th, that0, D, V, wq, Nx, N, scratch, ticket, out);
  SMC_LAUNCH_CHECK(c);
}

}  // namespace smc
