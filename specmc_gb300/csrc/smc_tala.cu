// The truncated anelastic liquid approximation (TALA) of the FP64 time step.
//
// The reference density rho_bar(z) = exp((1 - z) Di) (gamma = 1) enters in
// three places (specmc/physics/compressibility.py, core/rbc_galerkin.py:288-312):
//  * the velocity is the mass flux over rho_bar, u = curl(Psi) / rho_bar at the
//    CGL nodes (rbc_galerkin.py:355-372);
//  * the temperature equation weights the time derivative and the advection
//    by rho_bar (its Chebyshev product matrix Mrho), heats with rho_bar H and
//    adds the adiabatic term rho_bar u_z [1 - Di (1 - z + theta)]; its
//    per-wavenumber preconditioner is D2 - diag(k^2 + a0 rho_j)
//    (core/implicit_theta.py:159-178, :332-493);
//  * the coupled Stokes operator: Psi = G v with L^(rho) = D2 - a D - k^2
//    (a = -Di), the momentum block L2_i M = (D2 - 2a D + a^2 - k_i^2) M and
//    the commutator block A12 = sum c(a, k_i, k_j) D^p M D^q over the
//    monomials of stokes/stokes_tala.py:121-140, right-hand side
//    i k Ra rho_bar^2 theta, omega = -v / rho_bar (stokes/stokes_tala.py).
// The operator words are the same Chebyshev matrices the Boussinesq route
// uses; only their coefficients and two extra words (M D, D M) differ.
#include "smc_internal.cuh"
#include "smc_schur.cuh"
#include "smc_tala.cuh"

namespace smc {

// ------------------------------------------------------- small operators
__global__ void smc_tala_green_ops_kernel(const double* __restrict__ D, const double* __restrict__ D2,
                                          const double* __restrict__ kx, double a,
                                          double* __restrict__ Acm, int N) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  int p = blockIdx.y;
  int k = blockIdx.z;
  if (q >= N) return;
  double v;
  if (p == N - 2) v = (q & 1) ? -1.0 : 1.0;          // V[0] = T_q(-1)
  else if (p == N - 1) v = 1.0;                      // V[N-1] = T_q(1)
  else {
    const long long e = (long long)p * N + q;
    v = D2[e] - a * D[e];
    if (p == q) v -= kx[k] * kx[k];
  }
  Acm[(long long)k * N * N + (long long)q * N + p] = v;
}

void tala_green_ops(const Ctx& c, const double* D, const double* D2, const double* kx, double a,
                    double* Acm, int N, int Nk) {
  dim3 grd(ceil_div(N, 128), N, Nk);
  smc_tala_green_ops_kernel<<<grd, 128, 0, c.s>>>(D, D2, kx, a, Acm, N);
  SMC_LAUNCH_CHECK(c);
}

__global__ void smc_tala_theta_ops_kernel(const double* __restrict__ D2, const double* __restrict__ kx,
                                          double lam, const double* __restrict__ rho,
                                          double* __restrict__ Acm, int N) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  int p = blockIdx.y;
  int k = blockIdx.z;
  if (q >= N) return;
  double v;
  if (p == N - 2) v = (q & 1) ? -1.0 : 1.0;
  else if (p == N - 1) v = 1.0;
  else v = D2[(long long)p * N + q] - ((p == q) ? (kx[k] * kx[k] + lam * rho[p]) : 0.0);
  Acm[(long long)k * N * N + (long long)q * N + p] = v;
}

void tala_theta_ops(const Ctx& c, const double* D2, const double* kx, double lam, const double* rho,
                    double* Acm, int N, int Nk) {
  dim3 grd(ceil_div(N, 128), N, Nk);
  smc_tala_theta_ops_kernel<<<grd, 128, 0, c.s>>>(D2, kx, lam, rho, Acm, N);
  SMC_LAUNCH_CHECK(c);
}

// ------------------------------------------------- temperature equation
__global__ void smc_tala_theta_combine_kernel(const double2* __restrict__ v, const double2* __restrict__ A,
                                              const double* __restrict__ Mrho,
                                              const double* __restrict__ MrhoVi,
                                              const double* __restrict__ D2, const double* __restrict__ V,
                                              const double* __restrict__ kx, double a0,
                                              double2* __restrict__ out, int Nk, int N) {
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
    const double* Mr = Mrho + (long long)n * N;
    const double* Dr = D2 + (long long)n * N;
    const double* Wr = MrhoVi + (long long)n * N;
    const double2* Ak = A + (long long)k * N;
    double mr = 0, mi = 0, lr = 0, li = 0, ar = 0, ai = 0;
    for (int m = 0; m < N; ++m) {
      const double2 vm = vk[m], am = Ak[m];
      mr += Mr[m] * vm.x; mi += Mr[m] * vm.y;
      lr += Dr[m] * vm.x; li += Dr[m] * vm.y;
      ar += Wr[m] * am.x; ai += Wr[m] * am.y;
    }
    const double k2 = kx[k] * kx[k];
    const double2 vn = vk[n];
    lr -= k2 * vn.x; li -= k2 * vn.y;
    r = make_double2((a0 * mr - lr) - ar, (a0 * mi - li) - ai);
  }
  out[(long long)k * N + n] = r;
}

void tala_theta_combine(const Ctx& c, const double2* v, const double2* A, const double* Mrho,
                        const double* MrhoVi, const double* D2, const double* V, const double* kx,
                        double a0, double2* out, int Nk, int N) {
  dim3 grd(ceil_div(N, 128), Nk);
  smc_tala_theta_combine_kernel<<<grd, 128, 0, c.s>>>(v, A, Mrho, MrhoVi, D2, V, kx, a0, out, Nk, N);
  SMC_LAUNCH_CHECK(c);
}

__global__ void smc_tala_theta_rhs_kernel(const double2* __restrict__ th, const double2* __restrict__ prev,
                                          const double* __restrict__ Mrho, const double* __restrict__ rho_c,
                                          const double2* __restrict__ adiab, const double2* __restrict__ phi,
                                          double b0, double b1, double H, double2* __restrict__ b,
                                          int Nk, int N) {
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (n >= N || k >= Nk) return;
  const long long i = (long long)k * N + n;
  double2 v = make_double2(0.0, 0.0);
  if (n < N - 2) {
    const double* Mr = Mrho + (long long)n * N;
    const double2* tk = th + (long long)k * N;
    const double2* pk = prev + (long long)k * N;
    double sr = 0.0, si = 0.0;
    for (int m = 0; m < N; ++m) {
      double wr = b0 * tk[m].x, wi = b0 * tk[m].y;
      if (b1 != 0.0) { wr -= b1 * pk[m].x; wi -= b1 * pk[m].y; }
      sr += Mr[m] * wr; si += Mr[m] * wi;
    }
    v = make_double2(sr, si);
  }
  if (H != 0.0 && k == 0) v.x += H * rho_c[n];
  v = cadd(v, adiab[i]);
  if (phi && n < N - 2) v = cadd(v, phi[i]);
  b[i] = v;
}

void tala_theta_rhs(const Ctx& c, const double2* th, const double2* prev, const double* Mrho,
                    const double* rho_c, const double2* adiab, const double2* phi, double b0,
                    double b1, double H, double2* b, int Nk, int N) {
  dim3 grd(ceil_div(N, 128), Nk);
  smc_tala_theta_rhs_kernel<<<grd, 128, 0, c.s>>>(th, prev, Mrho, rho_c, adiab, phi, b0, b1, H, b,
                                                  Nk, N);
  SMC_LAUNCH_CHECK(c);
}

__global__ void smc_tala_adiabatic_kernel(const double* __restrict__ uz, const double* __restrict__ th,
                                          const double* __restrict__ rho, const double* __restrict__ z,
                                          double Di, double* __restrict__ out, long long npts, int N) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npts) return;
  const int j = (int)(i % N);
  const double br = 1.0 - Di * ((1.0 - z[j]) + th[i]);
  out[i] = (rho[j] * uz[i]) * br;
}

void tala_adiabatic_grid(const Ctx& c, const double* uz, const double* th, const double* rho,
                         const double* z, double Di, double* out, long long npts, int N) {
  smc_tala_adiabatic_kernel<<<ceil_div(npts, 256), 256, 0, c.s>>>(uz, th, rho, z, Di, out, npts, N);
  SMC_LAUNCH_CHECK(c);
}

__global__ void smc_grid_div_rho_kernel(double* __restrict__ ux, double* __restrict__ uz,
                                        const double* __restrict__ rho, long long npts, int N) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npts) return;
  const double r = rho[(int)(i % N)];
  ux[i] = ux[i] / r;
  uz[i] = uz[i] / r;
}

void grid_div_rho(const Ctx& c, double* ux, double* uz, const double* rho, long long npts, int N) {
  smc_grid_div_rho_kernel<<<ceil_div(npts, 256), 256, 0, c.s>>>(ux, uz, rho, npts, N);
  SMC_LAUNCH_CHECK(c);
}

__global__ void smc_scale_cols_kernel(const double2* __restrict__ in, const double* __restrict__ s,
                                      double alpha, double2* __restrict__ out, int Nk, int N) {
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (n >= N || k >= Nk) return;
  const long long i = (long long)k * N + n;
  out[i] = make_double2(alpha * (in[i].x * s[n]), alpha * (in[i].y * s[n]));
}

void scale_cols(const Ctx& c, const double2* in, const double* s, double alpha, double2* out,
                int Nk, int N) {
  dim3 grd(ceil_div(N, 128), Nk);
  smc_scale_cols_kernel<<<grd, 128, 0, c.s>>>(in, s, alpha, out, Nk, N);
  SMC_LAUNCH_CHECK(c);
}

// ------------------------------------------------------ Schur operator
// The A12 monomials (a_deriv, b_deriv, output-k power, input-k power, c(a))
// of stokes_tala.py:121-140, summed per word D^p M D^q at (ki, kj); the word
// order is W00 = M, W01 = M D, W02 = M D2, W10 = D M, W11 = D M D, W20 = D2 M.
__host__ __device__ inline void tala_a12_words(double a, double ki, double kj, double c[6]) {
  c[0] = ((-2.0 * a) * a) * ki * kj + ((2.0 * a) * a) * (kj * kj);
  c[1] = (-2.0 * a) * (ki * ki) + (4.0 * a) * ki * kj;
  c[2] = 2.0 * (ki * ki);
  c[3] = (2.0 * a) * ki * kj + (-4.0 * a) * (kj * kj);
  c[4] = -4.0 * ki * kj;
  c[5] = 2.0 * (kj * kj);
}

__global__ void smc_tala_schur_combine_kernel(const double2* __restrict__ t, const double2* __restrict__ T01,
                                              const double2* __restrict__ T02,
                                              const double2* __restrict__ T10,
                                              const double2* __restrict__ T11,
                                              const double2* __restrict__ T20,
                                              const double2* __restrict__ v, const double* __restrict__ D,
                                              const double* __restrict__ D2, const double* __restrict__ V,
                                              const double* __restrict__ kx, double a,
                                              double2* __restrict__ out, int Nk, int N) {
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (n >= N || k >= Nk) return;
  const long long o = (long long)k * N;
  double2 r;
  if (n >= N - 2) {
    const double* Vr = V + (n == N - 2 ? 0 : (long long)(N - 1) * N);
    double sr = 0, si = 0;
    for (int m = 0; m < N; ++m) { sr += v[o + m].x * Vr[m]; si += v[o + m].y * Vr[m]; }
    r = make_double2(sr, si);
  } else {
    // monomial coefficients c(a); the output-wavenumber powers are applied below
    const double c0011 = (-2.0 * a) * a, c0002 = (2.0 * a) * a, c0120 = -2.0 * a, c0111 = 4.0 * a,
                 c0220 = 2.0, c1011 = 2.0 * a, c1002 = -4.0 * a, c1111 = -4.0, c2002 = 2.0;
    const double kk = kx[k], k2 = kk * kk;
    const double* Dr = D + (long long)n * N;
    const double* D2r = D2 + (long long)n * N;
    double2 s2t = make_double2(0, 0), s1t = make_double2(0, 0);
    double2 s1p = make_double2(0, 0), s2p = make_double2(0, 0);
    for (int m = 0; m < N; ++m) {
      const double2 tm = t[o + m], a01 = T01[o + m], a02 = T02[o + m], a11 = T11[o + m];
      s2t.x += D2r[m] * tm.x; s2t.y += D2r[m] * tm.y;
      s1t.x += Dr[m] * tm.x;  s1t.y += Dr[m] * tm.y;
      // D^1 words: c1011 k T01 + c1002 T02 + c1111 k T11
      const double pr = c1011 * (kk * a01.x) + c1002 * a02.x + c1111 * (kk * a11.x);
      const double pi = c1011 * (kk * a01.y) + c1002 * a02.y + c1111 * (kk * a11.y);
      s1p.x += Dr[m] * pr; s1p.y += Dr[m] * pi;
      // D^2 word: c2002 T02
      s2p.x += D2r[m] * (c2002 * a02.x); s2p.y += D2r[m] * (c2002 * a02.y);
    }
    const double2 tn = t[o + n], b01 = T01[o + n], b02 = T02[o + n], b10 = T10[o + n],
                  b11 = T11[o + n], b20 = T20[o + n];
    const double aa = a * a - k2;
    double xr = (s2t.x - (2.0 * a) * s1t.x) + aa * tn.x;
    double xi = (s2t.y - (2.0 * a) * s1t.y) + aa * tn.y;
    // D^0 words
    const double p0r = c0011 * (kk * b01.x) + c0002 * b02.x + c0120 * (k2 * b10.x) +
                       c0111 * (kk * b11.x) + c0220 * (k2 * b20.x);
    const double p0i = c0011 * (kk * b01.y) + c0002 * b02.y + c0120 * (k2 * b10.y) +
                       c0111 * (kk * b11.y) + c0220 * (k2 * b20.y);
    r = make_double2(xr + ((p0r + s1p.x) + s2p.x), xi + ((p0i + s1p.y) + s2p.y));
  }
  out[o + n] = r;
}

void tala_schur_combine(const Ctx& c, const double2* t, const double2* T01, const double2* T02,
                        const double2* T10, const double2* T11, const double2* T20,
                        const double2* v, const double* D, const double* D2, const double* V,
                        const double* kx, double a, double2* out, int Nk, int N) {
  dim3 grd(ceil_div(N, 128), Nk);
  smc_tala_schur_combine_kernel<<<grd, 128, 0, c.s>>>(t, T01, T02, T10, T11, T20, v, D, D2, V, kx,
                                                      a, out, Nk, N);
  SMC_LAUNCH_CHECK(c);
}

// Block (i, j) of the dense TALA Schur matrix, column-major in A (n x n):
//   B = A11_d + (sum_w c_w(ki, kj) W_w[d]) G_j,   A11_d = W20 - 2a W10 + (a^2 - ki^2) W00
// at the shift d = i - j, minus, for j >= 1 and i + j < Nk, the partner half
// at the shift i + j with the coefficients at (ki, -kj).  Tau rows N-2, N-1:
// v(0), v(1) on the diagonal block, zero elsewhere.  Same tiling as the
// Boussinesq block kernel: 32 x 32 output tile, 256 threads, 2 x 2 per thread.
__global__ void smc_tala_block_kernel(const double2* __restrict__ W00, const double2* __restrict__ W01,
                                      const double2* __restrict__ W02, const double2* __restrict__ W10,
                                      const double2* __restrict__ W11, const double2* __restrict__ W20,
                                      const double* __restrict__ G, const double* __restrict__ V,
                                      const double* __restrict__ kx, double a,
                                      double2* __restrict__ A, int Nk, int N) {
  __shared__ double2 Ts[32][33];
  __shared__ double Gs[32][33];
  const int blk = blockIdx.z;
  const int i = blk / Nk, j = blk % Nk;
  const int p0 = blockIdx.y * 32, r0 = blockIdx.x * 32;
  const long long n = (long long)Nk * N;
  const long long NN = (long long)N * N;
  const double ki = kx[i], kj = kx[j];
  const long long od = (long long)(i - j + Nk - 1) * NN;
  const bool part = (j >= 1) && (i + j < Nk);
  const long long op = (long long)(i + j + Nk - 1) * NN;
  double cd[6], cp[6];
  tala_a12_words(a, ki, kj, cd);
  tala_a12_words(a, ki, -kj, cp);
  const double a11_1 = -2.0 * a, a11_0 = a * a - ki * ki;
  const int tp = threadIdx.x % 16, tr = threadIdx.x / 16;
  double2 acc[2][2] = {{{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}};
  const double* Gj = G + (long long)j * NN;
  for (int k0 = 0; k0 < N; k0 += 32) {
    for (int t = threadIdx.x; t < 1024; t += 256) {
      const int pp = t / 32, kk = t % 32;
      const int gp = p0 + pp, gk = k0 + kk;
      double2 tv = make_double2(0.0, 0.0);
      if (gp < N && gk < N) {
        const long long e = (long long)gp * N + gk;
        const double2 w[6] = {W00[od + e], W01[od + e], W02[od + e],
                              W10[od + e], W11[od + e], W20[od + e]};
        for (int q = 0; q < 6; ++q) { tv.x += cd[q] * w[q].x; tv.y += cd[q] * w[q].y; }
        if (part) {
          const double2 u[6] = {W00[op + e], W01[op + e], W02[op + e],
                                W10[op + e], W11[op + e], W20[op + e]};
          for (int q = 0; q < 6; ++q) { tv.x -= cp[q] * u[q].x; tv.y -= cp[q] * u[q].y; }
        }
      }
      Ts[pp][kk] = tv;
      const int gk2 = k0 + pp, gr = r0 + kk;
      Gs[pp][kk] = (gk2 < N && gr < N) ? Gj[(long long)gk2 * N + gr] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < 32; ++kk) {
      const double2 t0 = Ts[tp * 2][kk], t1 = Ts[tp * 2 + 1][kk];
      const double g0 = Gs[kk][tr * 2], g1 = Gs[kk][tr * 2 + 1];
      acc[0][0].x += t0.x * g0; acc[0][0].y += t0.y * g0;
      acc[0][1].x += t0.x * g1; acc[0][1].y += t0.y * g1;
      acc[1][0].x += t1.x * g0; acc[1][0].y += t1.y * g0;
      acc[1][1].x += t1.x * g1; acc[1][1].y += t1.y * g1;
    }
    __syncthreads();
  }
  for (int b = 0; b < 2; ++b)
    for (int q = 0; q < 2; ++q) {
      const int gp = p0 + tp * 2 + q, gr = r0 + tr * 2 + b;
      if (gp >= N || gr >= N) continue;
      const long long e = (long long)gp * N + gr;
      double2 v;
      if (gp >= N - 2) {
        const double bc = (i == j) ? V[(gp == N - 2 ? 0 : (long long)(N - 1) * N) + gr] : 0.0;
        v = make_double2(bc, 0.0);
      } else {
        const double2 m20 = W20[od + e], m10 = W10[od + e], m00 = W00[od + e];
        v = make_double2(m20.x + a11_1 * m10.x + a11_0 * m00.x + acc[q][b].x,
                         m20.y + a11_1 * m10.y + a11_0 * m00.y + acc[q][b].y);
        if (part) {
          const double2 n20 = W20[op + e], n10 = W10[op + e], n00 = W00[op + e];
          v.x -= n20.x + a11_1 * n10.x + a11_0 * n00.x;
          v.y -= n20.y + a11_1 * n10.y + a11_0 * n00.y;
        }
      }
      A[((long long)i * N + gp) + ((long long)j * N + gr) * n] = v;
    }
}

void assemble_schur_tala(const Ctx& c, const double2* Md, const double* D, const double* D2,
                         const double* G, const double* V, const double* kx, double a,
                         double2* A, int Nk, int N, double2* work) {
  if ((long long)Nk * Nk > 65535)
    throw std::runtime_error("dense TALA Schur assembly: Nk^2 blocks exceed the launch grid");
  const long long NN = (long long)N * N;
  const int nd = 2 * Nk - 1;
  double2* W20 = work;             // D2 M_d
  double2* W02 = W20 + nd * NN;    // M_d D2
  double2* W01 = W02 + nd * NN;    // M_d D
  double2* W11 = W01 + nd * NN;    // D M_d D
  double2* W10 = W11 + nd * NN;    // D M_d
  bgemm(c, false, D2, 0, true, Md, NN, W20, NN, N, nd, 1.0);
  bgemm(c, true, Md, NN, false, D2, 0, W02, NN, N, nd, 1.0);
  bgemm(c, true, Md, NN, false, D, 0, W01, NN, N, nd, 1.0);
  bgemm(c, false, D, 0, true, W01, NN, W11, NN, N, nd, 1.0);
  bgemm(c, false, D, 0, true, Md, NN, W10, NN, N, nd, 1.0);
  dim3 grd(ceil_div(N, 32), ceil_div(N, 32), Nk * Nk);
  smc_tala_block_kernel<<<grd, 256, 0, c.s>>>(Md, W01, W02, W10, W11, W20, G, V, kx, a, A, Nk, N);
  SMC_LAUNCH_CHECK(c);
}

}  // namespace smc
