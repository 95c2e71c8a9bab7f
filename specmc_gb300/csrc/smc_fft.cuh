// Radix-2 FFT in shared memory, used by the x-direction convolutions of the
// pseudo-spectral mult_eta (plain form), of the fused Schur operator and of
// the Krylov engine (fast form).  Their x-grid length L is a power of two
// chosen >= 3 Nk - 2, the length at which the product of two Nk-mode
// fields is reproduced without aliasing.
#pragma once

namespace smc {

// In-place FFT of a[0..L), L = 2^logL, by threads t = 0..nt-1 of a thread
// group; every group of the CTA calls it together (the stages are separated
// by __syncthreads).  dir = +1: a_k <- sum_j a_j e^{+2 pi i jk/L}; dir = -1:
// e^{-2 pi i jk/L}.  tw[m] = e^{+2 pi i m/L} for m < L/2.  Natural order in
// and out: the input is first permuted to bit-reversed order, then log2 L
// decimation-in-time butterfly stages run.
template <class C>
__device__ __forceinline__ void cta_fft(C* a, int L, int logL, const C* tw, int dir, int t, int nt) {
  for (int i = t; i < L; i += nt) {
    const int r = (int)(__brev((unsigned)i) >> (32 - logL));
    if (r > i) {
      const C x = a[i];
      a[i] = a[r];
      a[r] = x;
    }
  }
  __syncthreads();
  for (int half = 1, step = L >> 1; half < L; half <<= 1, step >>= 1) {
    for (int q = t; q < (L >> 1); q += nt) {
      const int pos = q & (half - 1);
      const int i0 = ((q - pos) << 1) + pos;      // (q / half) 2 half + pos
      const int i1 = i0 + half;
      C w = tw[pos * step];
      if (dir < 0) w.y = -w.y;
      const C u = a[i0], v0 = a[i1];
      C v;
      v.x = v0.x * w.x - v0.y * w.y;
      v.y = v0.x * w.y + v0.y * w.x;
      C o0, o1;
      o0.x = u.x + v.x; o0.y = u.y + v.y;
      o1.x = u.x - v.x; o1.y = u.y - v.y;
      a[i0] = o0;
      a[i1] = o1;
    }
    __syncthreads();
  }
}

// The same transform by the 32 lanes of one warp on its own row a[0..L):
// the same butterflies (so the same values), the stages separated by
// __syncwarp instead of CTA barriers, so the warps of a CTA run independent
// transforms side by side.
template <class C>
__device__ __forceinline__ void warp_fft(C* a, int L, int logL, const C* tw, int dir, int lane) {
  for (int i = lane; i < L; i += 32) {
    const int r = (int)(__brev((unsigned)i) >> (32 - logL));
    if (r > i) {
      const C x = a[i];
      a[i] = a[r];
      a[r] = x;
    }
  }
  __syncwarp();
  for (int half = 1, step = L >> 1; half < L; half <<= 1, step >>= 1) {
    for (int q = lane; q < (L >> 1); q += 32) {
      const int pos = q & (half - 1);
      const int i0 = ((q - pos) << 1) + pos;
      const int i1 = i0 + half;
      C w = tw[pos * step];
      if (dir < 0) w.y = -w.y;
      const C u = a[i0], v0 = a[i1];
      C v;
      v.x = v0.x * w.x - v0.y * w.y;
      v.y = v0.x * w.y + v0.y * w.x;
      C o0, o1;
      o0.x = u.x + v.x; o0.y = u.y + v.y;
      o1.x = u.x - v.x; o1.y = u.y - v.y;
      a[i0] = o0;
      a[i1] = o1;
    }
    __syncwarp();
  }
}

// the engine's Schur x-convolution runs one transform per warp (4 fields x 2
// z-points per CTA of 8 warps) when the 8 rows and the twiddles fit this
// budget of shared memory, else one per 64-thread group (4 fields, one
// z-point at a time)
__host__ __device__ __forceinline__ bool schur_x_by_warp(int L, int csize) {
  return (long long)(L / 2 + 8 * L) * csize <= 64 * 1024;
}

// log2 of a power of two
__device__ __forceinline__ int ilog2_pow2(int L) { return __ffs(L) - 1; }

}  // namespace smc
