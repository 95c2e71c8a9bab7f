// The trailing update of the dense complex LU (A22 -= L21 U12, one 32-column
// panel at a time) on the tensor cores, with FP64 accuracy.
//
// The plain form's lagged Schur factor (stokes/lagged_stokes.py:274-300:
// sla.lu_factor of the (Nk Nz)^2 complex Schur matrix) spends ~3/4 of its
// time in this update, which on GB300's FP64 pipe runs at ~1 TFLOP/s.  The
// update is a complex GEMM with K = 32, written as two real GEMMs with
// K = 64 that share one operand:
//     Re C = [Lr  Li] . [Ur ; -Ui],      Im C = [Lr  Li] . [Ui ; Ur],
// and each real GEMM is formed by Ozaki's error-free splitting, as the
// z-contractions of smc_tc.cu: every row of [Lr Li] and every column of
// [Ur ; Ui] is scaled by a power of two into (-1, 1) and cut into eight 7-bit
// slices (integers in [-127, 127], exact in bf16); the products of one level
// p + q -- at most 8 slice pairs of K = 64 terms, below 8 * 64 * 127^2 < 2^24
// -- accumulate exactly in FP32 in tensor memory; the 8 levels are combined in
// a 64-bit integer in units of 2^-52 of the scales, converted once, scaled
// and subtracted from A22 in FP64.  The result equals the FP64 update to
// roundoff (about 2^-52 of the row and column scales).
//
// Per panel: one kernel cuts L21 into slices (a 128-row tile image per CTA),
// one cuts U12 (a 32-column tile image, both sign arrangements), both written
// in the exact shared-memory image of the MMA operands; then each CTA of the
// update kernel brings its two images in by bulk copies (cp.async.bulk onto
// one mbarrier, 192 KB), one thread issues the 288 MMAs (36 slice pairs x 4
// k-steps x Re/Im) into 16 accumulators of 32 columns (all 512 TMEM
// columns), commits them to a second mbarrier, and the CTA's four warps read
// their 32 rows back, combine, scale and update A22 in place (column-major:
// consecutive lanes touch consecutive rows).  Every mbarrier wait is bounded;
// on time-out the CTA leaves A22 untouched, flags an error the host raises,
// and still frees its tensor memory.
#include <cuda_bf16.h>

#include "smc_tc.cuh"

namespace smc {

namespace {

constexpr int LU_M = 128;                 // rows of A22 per CTA (TMEM lanes)
constexpr int LU_N = 32;                  // columns of A22 per CTA
constexpr int LU_K = 64;                  // [Lr Li] / [Ur ; Ui]: 2 x the panel width 32
constexpr int LU_SL = 8;                  // slices
constexpr int LU_A_SLICE = LU_M * LU_K * 2;            // 16 KB
constexpr int LU_B_SLICE = LU_N * LU_K * 2;            // 4 KB
constexpr int LU_A_TILE = LU_SL * LU_A_SLICE;          // 128 KB
constexpr int LU_B_TILE = 2 * LU_SL * LU_B_SLICE;      // 64 KB (Re and Im arrangements)
constexpr int LU_SMEM = LU_A_TILE + LU_B_TILE;         // 192 KB: one CTA per SM
constexpr int LU_THREADS = 128;
constexpr long long LU_WAIT_NS = 200000000LL;
constexpr int LU_COPY = 16384;                          // bytes per bulk copy

__device__ __forceinline__ uint32_t s_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return (long long)t;
}
__device__ bool bar_wait(uint32_t bar, uint32_t phase) {
  const long long t0 = now_ns();
  for (int i = 0;; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok) : "r"(bar), "r"(phase) : "memory");
    if (ok) return true;
    if ((i & 63) == 63 && now_ns() - t0 > LU_WAIT_NS) return false;
  }
}
// K-major core matrices (8 rows x 16 bytes) of a 64-wide K: core (row / 8,
// k / 8) at ((row / 8) * 8 + k / 8) * 128 -- LBO 128 B (next along K), SBO
// 1024 B (next 8 rows)
__device__ __forceinline__ int lu_off(int row, int k) {
  return (((row >> 3) * 8 + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1);
}
__device__ __forceinline__ uint64_t lu_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) |
         ((uint64_t)(1024 >> 4) << 32) | (1ull << 46);
}
constexpr uint32_t LU_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(LU_N >> 3) << 17) |
                              ((uint32_t)(LU_M >> 4) << 24);

// trunc(|x| 2^(56 - e)) for |x| < 2^e (integer ops on the bit pattern)
__device__ __forceinline__ unsigned long long fix56(double x, int e, bool* neg) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  *neg = (b >> 63) != 0;
  const int ex = (int)((b >> 52) & 0x7ff);
  unsigned long long m = b & ((1ull << 52) - 1);
  int sh;
  if (ex == 0) sh = -1074 + 56 - e;
  else { m |= 1ull << 52; sh = ex - 1075 + 56 - e; }
  if (sh >= 0) return m << sh;
  return sh > -64 ? (m >> (-sh)) : 0ull;
}
__device__ __forceinline__ unsigned short bf16i(unsigned s, bool neg) {
  if (s == 0) return 0;
  const int msb = 31 - __clz(s);
  return (unsigned short)(((unsigned)neg << 15) | ((unsigned)(127 + msb) << 7) |
                          ((s << (7 - msb)) & 0x7fu));
}
__device__ __forceinline__ int exp_above(double amax) {   // amax < 2^e
  int e = 0;
  if (amax > 0.0) frexp(amax, &e);
  return e;
}

// L21 slices: CTA = one 128-row tile, thread = one row; [Lr Li] of the row
__global__ void __launch_bounds__(LU_M) smc_tclu_slice_a_kernel(
    const double2* __restrict__ A, int n, int p0, int nbp, unsigned char* __restrict__ img,
    int* __restrict__ rexp) {
  const int r0 = p0 + nbp, row = threadIdx.x;
  const int gr = r0 + blockIdx.x * LU_M + row;
  const bool ok = gr < n;
  double2 v[32];
  double amax = 0.0;
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    v[k] = (ok && k < nbp) ? A[gr + (long long)(p0 + k) * n] : make_double2(0.0, 0.0);
    amax = fmax(amax, fmax(fabs(v[k].x), fabs(v[k].y)));
  }
  const int e = exp_above(amax);
  rexp[blockIdx.x * LU_M + row] = e;
  unsigned char* t = img + (long long)blockIdx.x * LU_A_TILE;
  for (int kb = 0; kb < LU_K / 8; ++kb) {
    unsigned short sl[LU_SL][8];
    for (int i = 0; i < 8; ++i) {
      const int k = kb * 8 + i;                     // 0..31 Re, 32..63 Im
      const double x = k < 32 ? v[k].x : v[k - 32].y;
      bool neg;
      const unsigned long long u = fix56(x, e, &neg);
      for (int p = 0; p < LU_SL; ++p) sl[p][i] = bf16i((unsigned)((u >> (49 - 7 * p)) & 127u), neg);
    }
    const int off = lu_off(row, kb * 8);
    for (int p = 0; p < LU_SL; ++p) {
      uint4 w;
      w.x = (uint32_t)sl[p][0] | ((uint32_t)sl[p][1] << 16);
      w.y = (uint32_t)sl[p][2] | ((uint32_t)sl[p][3] << 16);
      w.z = (uint32_t)sl[p][4] | ((uint32_t)sl[p][5] << 16);
      w.w = (uint32_t)sl[p][6] | ((uint32_t)sl[p][7] << 16);
      *reinterpret_cast<uint4*>(t + p * LU_A_SLICE + off) = w;
    }
  }
}

// U12 slices: CTA = one 32-column tile, thread = one column (lanes of one
// warp); image: 8 slices of [Ur ; -Ui] (Re), then 8 of [Ui ; Ur] (Im)
__global__ void __launch_bounds__(LU_N) smc_tclu_slice_b_kernel(
    const double2* __restrict__ A, int n, int p0, int nbp, unsigned char* __restrict__ img,
    int* __restrict__ cexp) {
  const int c0 = p0 + nbp, col = threadIdx.x;
  const int gc = c0 + blockIdx.x * LU_N + col;
  const bool ok = gc < n;
  double2 v[32];
  double amax = 0.0;
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    v[k] = (ok && k < nbp) ? A[(p0 + k) + (long long)gc * n] : make_double2(0.0, 0.0);
    amax = fmax(amax, fmax(fabs(v[k].x), fabs(v[k].y)));
  }
  const int e = exp_above(amax);
  cexp[blockIdx.x * LU_N + col] = e;
  unsigned char* t = img + (long long)blockIdx.x * LU_B_TILE;
  for (int kb = 0; kb < LU_K / 8; ++kb) {
    unsigned short sr[LU_SL][8], si[LU_SL][8];
    for (int i = 0; i < 8; ++i) {
      const int k = kb * 8 + i;
      // Re arrangement: Ur (k < 32), -Ui; Im arrangement: Ui (k < 32), Ur
      const double xr = k < 32 ? v[k].x : -v[k - 32].y;
      const double xi = k < 32 ? v[k].y : v[k - 32].x;
      bool nr, ni;
      const unsigned long long ur = fix56(xr, e, &nr), ui = fix56(xi, e, &ni);
      for (int p = 0; p < LU_SL; ++p) {
        sr[p][i] = bf16i((unsigned)((ur >> (49 - 7 * p)) & 127u), nr);
        si[p][i] = bf16i((unsigned)((ui >> (49 - 7 * p)) & 127u), ni);
      }
    }
    const int off = lu_off(col, kb * 8);
    for (int p = 0; p < LU_SL; ++p) {
      uint4 w;
      w.x = (uint32_t)sr[p][0] | ((uint32_t)sr[p][1] << 16);
      w.y = (uint32_t)sr[p][2] | ((uint32_t)sr[p][3] << 16);
      w.z = (uint32_t)sr[p][4] | ((uint32_t)sr[p][5] << 16);
      w.w = (uint32_t)sr[p][6] | ((uint32_t)sr[p][7] << 16);
      *reinterpret_cast<uint4*>(t + p * LU_B_SLICE + off) = w;
      w.x = (uint32_t)si[p][0] | ((uint32_t)si[p][1] << 16);
      w.y = (uint32_t)si[p][2] | ((uint32_t)si[p][3] << 16);
      w.z = (uint32_t)si[p][4] | ((uint32_t)si[p][5] << 16);
      w.w = (uint32_t)si[p][6] | ((uint32_t)si[p][7] << 16);
      *reinterpret_cast<uint4*>(t + (LU_SL + p) * LU_B_SLICE + off) = w;
    }
  }
}

__global__ void __launch_bounds__(LU_THREADS, 1) smc_tclu_gemm_kernel(
    double2* __restrict__ A, int n, int p0, int nbp, const unsigned char* __restrict__ aimg,
    const int* __restrict__ rexp, const unsigned char* __restrict__ bimg,
    const int* __restrict__ cexp, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* sA = sm;
  unsigned char* sB = sm + LU_A_TILE;
  __shared__ __align__(8) unsigned long long bar_cp, bar_mma;
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail;
  const int t = threadIdx.x, warp = t >> 5;
  const int mt = blockIdx.y, nt = blockIdx.x;
  const uint32_t bcp = s_u32(&bar_cp), bmm = s_u32(&bar_mma);
  if (t == 0) {
    s_fail = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bcp) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bmm) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     s_u32(&tmem_base)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  if (t == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bcp),
                 "r"(LU_SMEM)
                 : "memory");
    const unsigned char* ga = aimg + (long long)mt * LU_A_TILE;
    const unsigned char* gb = bimg + (long long)nt * LU_B_TILE;
    for (int o = 0; o < LU_A_TILE; o += LU_COPY)
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
              "r"(s_u32(sA + o)),
          "l"(ga + o), "r"(LU_COPY), "r"(bcp)
          : "memory");
    for (int o = 0; o < LU_B_TILE; o += LU_COPY)
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
              "r"(s_u32(sB + o)),
          "l"(gb + o), "r"(LU_COPY), "r"(bcp)
          : "memory");
    if (!bar_wait(bcp, 0)) s_fail = 1;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!s_fail) {
      bool seen[2 * LU_SL];
      for (int i = 0; i < 2 * LU_SL; ++i) seen[i] = false;
      for (int p = 0; p < LU_SL; ++p)
        for (int q = 0; p + q < LU_SL; ++q)
          for (int part = 0; part < 2; ++part) {      // 0: Re, 1: Im
            const int acc_i = part * LU_SL + p + q;
            for (int ks = 0; ks < LU_K / 16; ++ks) {
              const uint64_t ad = lu_desc(s_u32(sA + p * LU_A_SLICE + ks * 256));
              const uint64_t bd = lu_desc(s_u32(sB + (part * LU_SL + q) * LU_B_SLICE + ks * 256));
              const uint32_t en = seen[acc_i] ? 1u : 0u;
              asm volatile(
                  "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                  " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
                      tmem + (uint32_t)(acc_i * LU_N)),
                  "l"(ad), "l"(bd), "r"(LU_IDESC), "r"(en)
                  : "memory");
              seen[acc_i] = true;
            }
          }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     bmm)
                 : "memory");
  }
  __syncthreads();
  if (!bar_wait(bmm, 0)) s_fail = 1;
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const bool failed = s_fail != 0;
  if (failed) {
    bar_wait(bmm, 0);
    if (t == 0) atomicExch(err, 1);
  }
  // epilogue: lane = row 32 warp + lane of the tile; 2 groups of 16 columns
  const int row = 32 * warp + (t & 31);
  const int gr = p0 + nbp + mt * LU_M + row;
  const int er = rexp[mt * LU_M + row];
  for (int cg = 0; cg < LU_N / 16; ++cg) {
    long long acc[2][16];
    for (int part = 0; part < 2; ++part) {
      for (int j = 0; j < 16; ++j) acc[part][j] = 0;
      for (int lv = LU_SL - 1; lv >= 0; --lv) {
        uint32_t v[16];
        const uint32_t ta = tmem + ((uint32_t)(32 * warp) << 16) +
                            (uint32_t)((part * LU_SL + lv) * LU_N + cg * 16);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
            "%11, %12, %13, %14, %15}, [%16];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
              "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
              "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(ta)
            : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        for (int j = 0; j < 16; ++j) {
          const long long d = (long long)__float2int_rz(__uint_as_float(v[j]));
          acc[part][j] += lv <= 5 ? (d << (38 - 7 * lv)) : (d >> (7 * lv - 38));
        }
      }
    }
    if (!failed && gr < n) {
      for (int j = 0; j < 16; ++j) {
        const int cc = nt * LU_N + cg * 16 + j;
        const int gc = p0 + nbp + cc;
        if (gc >= n) continue;
        const double sc = ldexp(1.0, er + cexp[cc] - 52);
        double2* e = &A[gr + (long long)gc * n];
        double2 x = *e;
        x.x -= __ll2double_rn(acc[0][j]) * sc;
        x.y -= __ll2double_rn(acc[1][j]) * sc;
        *e = x;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512)
                 : "memory");
}

}  // namespace

size_t tclu_work_bytes(int n) {
  const long long mt = ceil_div(n, LU_M), nt = ceil_div(n, LU_N);
  return (size_t)mt * LU_A_TILE + (size_t)nt * LU_B_TILE + (size_t)(mt * LU_M + nt * LU_N) * 4 + 1024;
}

void tclu_update(const Ctx& c, double2* A, int n, int p0, int nbp, void* work, int* err) {
  const int rest = n - p0 - nbp;
  if (rest <= 0) return;
  if (nbp > 32) throw std::runtime_error("tclu_update: panel wider than 32");
  const int mt = ceil_div(rest, LU_M), nt = ceil_div(rest, LU_N);
  unsigned char* aimg = static_cast<unsigned char*>(work);
  unsigned char* bimg = aimg + (size_t)ceil_div(n, LU_M) * LU_A_TILE;
  int* rexp = reinterpret_cast<int*>(bimg + (size_t)ceil_div(n, LU_N) * LU_B_TILE);
  int* cexp = rexp + ceil_div(n, LU_M) * LU_M;
  smc_tclu_slice_a_kernel<<<mt, LU_M, 0, c.s>>>(A, n, p0, nbp, aimg, rexp);
  SMC_LAUNCH_CHECK(c);
  smc_tclu_slice_b_kernel<<<nt, LU_N, 0, c.s>>>(A, n, p0, nbp, bimg, cexp);
  SMC_LAUNCH_CHECK(c);
  static bool attr = false;
  if (!attr) {
    SMC_CUDA(cudaFuncSetAttribute((const void*)smc_tclu_gemm_kernel,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, LU_SMEM));
    attr = true;
  }
  smc_tclu_gemm_kernel<<<dim3(nt, mt), LU_THREADS, LU_SMEM, c.s>>>(A, n, p0, nbp, aimg, rexp, bimg,
                                                                   cexp, err);
  SMC_LAUNCH_CHECK(c);
}

}  // namespace smc
