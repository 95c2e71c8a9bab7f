// z-contractions of the Fourier x Chebyshev transforms on the tensor cores
// (tcgen05), with FP64 accuracy.
//
// The contraction Y[k][n] = f(k) sum_m Z[n][m] X[k][m] of the spectral
// transforms (core/rbc_galerkin.py:322-340: the Chebyshev V, V^-1, D, D^2
// products of grid / coeffs / _synth_pad / _trunc_pad) is a real GEMM:
// C[r][n] = sum_m A[r][m] B[n][m] with A the 2 Nk rows (Re, Im per mode k) of
// X and B = Z, both K-major (m contiguous).  GB300's FP64 pipe runs ~1/60 of
// its FP32 rate, while its bf16 tensor cores run three orders of magnitude
// above FP64, so the product is formed by Ozaki's error-free splitting
// (Ozaki, Ogita, Oishi, Rump, Numer. Algorithms 59 (2012)):
//
//   * every row of A and of B is scaled by a power of two so that its
//     entries lie in (-1, 1), and cut into TC_SLICES slices of 7 bits each:
//     a = sum_p s_p 2^(-7p), s_p an integer in [-127, 127] -- exact in bf16;
//   * the product of slices p and q is a sum of K <= 128 integer products of
//     at most 14 bits (|s| <= 127), and the products of one level L = p + q
//     (at most 8 of them) sum to at most 8 * 128 * 127^2 = 16,516,096 <
//     2^24: every partial sum is an integer below 2^24, which the FP32
//     accumulator holds exactly, so the tensor cores return each level
//     exactly;
//   * the levels L = 2 .. TC_SLICES + 1 (the products whose weight reaches
//     2^-63 relative to the row scales) are combined in 64-bit integers,
//     sum_L D_L 2^(52 - 7 L) (the two lowest levels shifted right; |D_L| <
//     2^24, so the sum stays below 2^62.01), converted to FP64 once and
//     scaled back with one FP64 product: C = 2^(e_r + f_n - 52) x that sum.
//
// The dropped terms, the operands' own 56-bit truncation and the bits
// dropped in the combination leave an error of about 2^-52 of the row and
// column scales -- the size of the FP64 SIMT contraction's own rounding, so
// the result is as accurate as the contraction it replaces (both are
// compared with the oracle in the tests).  The slices are cut with integer
// arithmetic on the FP64 bit patterns (GB300's FP64 pipe is its narrowest
// unit), so the only FP64 work is one conversion and one product per output.
//
// One CTA forms a 128 x 32 tile of C for every level in tensor memory (8
// accumulators of 32 FP32 columns: 256 TMEM columns, two CTAs per SM).  The
// operator's slices (B) are split once and stored in the exact shared-memory
// image of the MMA operand, so each 32-wide K chunk of a tile arrives in one
// bulk copy (cp.async.bulk, the TMA's non-tensor form, completing on an
// mbarrier); the data's slices (A) are cut by the CTA's threads while the
// copy is in flight.  One thread issues the MMAs (tcgen05.mma kind::f16,
// bf16 operands, FP32 accumulators in TMEM) and commits them to a second
// mbarrier; every wait on an mbarrier is bounded, after which the CTA flags
// an error, writes NaN and still frees its tensor memory.
#include <cuda_bf16.h>

#include "smc_tc.cuh"

namespace smc {

namespace {

constexpr int TC_THREADS = 128;
constexpr int TC_SMEM = TC_SLICES * (TC_A_SLICE_BYTES + TC_B_SLICE_BYTES);   // 80 KB: 2 CTAs per SM
constexpr int TC_TMEM_COLS = 256;                                         // 2 x 256 = the SM's 512
constexpr long long TC_WAIT_NS = 200000000LL; // 0.2 s: the MMAs of a tile take microseconds

struct TcJob {
  const double2* X = nullptr;
  double2* Y = nullptr;
  const void* bslices = nullptr;   // TcOperator::slices
  const double* bscale = nullptr;  // TcOperator::scale
  KFactor f;
  int accumulate = 0, x_real = 0, zero_tau = 0;
};
struct TcJobs4 { TcJob j[4]; };

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ long long tc_now() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return (long long)t;
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok) : "r"(bar), "r"(phase) : "memory");
  return ok != 0;
}
// bounded wait on phase `phase` of the mbarrier; false after TC_WAIT_NS
__device__ bool mbar_wait(uint32_t bar, uint32_t phase) {
  const long long t0 = tc_now();
  for (int i = 0;; ++i) {
    if (mbar_try(bar, phase)) return true;
    if ((i & 63) == 63 && tc_now() - t0 > TC_WAIT_NS) return false;
  }
}

// shared-memory matrix descriptor of tcgen05 (no swizzle, K-major core
// matrices of 8 rows x 16 bytes): start address, leading byte offset (next
// core matrix along K), stride byte offset (next 8-row group), version 1
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), bf16
// A and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at 24
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TC_N >> 3) << 17) |
                              ((uint32_t)(TC_M >> 4) << 24);

// byte offset of element (row, kk) of a K-major tile of 32-wide K chunks:
// core matrix (row / 8, kk / 8) at ((row / 8) * 4 + kk / 8) * 128, row % 8
// at 16 bytes, kk % 8 at 2 bytes -- LBO 128, SBO 512
__host__ __device__ __forceinline__ int tc_off(int row, int kk) {
  return (((row >> 3) * 4 + (kk >> 3)) << 7) + ((row & 7) << 4) + ((kk & 7) << 1);
}

__device__ __forceinline__ unsigned short bf16_bits(double v) {
  const __nv_bfloat16 h = __float2bfloat16_rn((float)v);   // |v| <= 127, an integer: exact
  return *reinterpret_cast<const unsigned short*>(&h);
}

// trunc(|x| 2^(56 - e)) for |x| < 2^e, from the bit pattern (integer ops);
// *neg = sign of x
__device__ __forceinline__ unsigned long long fixed56(double x, int e, bool* neg) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  *neg = (b >> 63) != 0;
  const int ex = (int)((b >> 52) & 0x7ff);
  unsigned long long m = b & ((1ull << 52) - 1);
  int sh;
  if (ex == 0) sh = -1074 + 56 - e;                 // subnormal: m 2^-1074
  else { m |= 1ull << 52; sh = ex - 1075 + 56 - e; }
  if (sh >= 0) return m << sh;                       // sh <= 3 since |x| < 2^e
  return sh > -64 ? (m >> (-sh)) : 0ull;
}

// bf16 bit pattern of the integer +-s, 0 <= s <= 127 (exact)
__device__ __forceinline__ unsigned short bf16_int(unsigned s, bool neg) {
  if (s == 0) return 0;
  const int msb = 31 - __clz(s);
  return (unsigned short)(((unsigned)neg << 15) | ((unsigned)(127 + msb) << 7) |
                          ((s << (7 - msb)) & 0x7fu));
}

// B operator split: one warp per row q (rows padded to ntiles * TC_N stay zero)
__global__ void smc_tc_pack_kernel(const double* __restrict__ Z, int rows, int K, int nchunks,
                                   unsigned char* __restrict__ out, double* __restrict__ scale) {
  const int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= rows) return;
  const double* zr = Z + (long long)q * K;
  double mx = 0.0;
  for (int m = lane; m < K; m += 32) mx = fmax(mx, fabs(zr[m]));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  int e = 0;
  if (mx > 0.0) frexp(mx, &e);                       // mx < 2^e
  if (lane == 0) scale[q] = ldexp(1.0, e);
  const int tile = q / TC_N, row = q % TC_N;
  for (int m = lane; m < K; m += 32) {
    double a = ldexp(zr[m], -e);                     // exact: |a| < 1
    unsigned char* blk = out + ((long long)tile * nchunks + m / TC_KC) * TC_B_CHUNK_BYTES;
    const int off = tc_off(row, m % TC_KC);
    for (int p = 0; p < TC_SLICES; ++p) {
      const double t = a * 128.0;
      const double s = trunc(t);
      a = t - s;
      *reinterpret_cast<unsigned short*>(blk + p * TC_B_SLICE_BYTES + off) = bf16_bits(s);
    }
  }
}

__global__ void __launch_bounds__(TC_THREADS, 2) smc_tc_zmat_kernel(
    const __grid_constant__ TcJobs4 jobs, int Nk, int N, int nchunks,
    const double* __restrict__ kx, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* sA = sm;                                  // TC_SLICES x 8 KB
  unsigned char* sB = sm + TC_SLICES * TC_A_SLICE_BYTES;   // TC_SLICES x 4 KB
  static_assert(TC_SLICES * (TC_A_SLICE_BYTES + TC_B_SLICE_BYTES) <= TC_SMEM, "tiles exceed smem");
  static_assert(TC_SLICES * TC_N <= TC_TMEM_COLS, "levels exceed tensor memory");
  __shared__ __align__(8) unsigned long long bar_tma, bar_mma;
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail;
  const TcJob& jb = jobs.j[blockIdx.z];
  const int t = threadIdx.x, warp = t >> 5;
  const int m0 = blockIdx.x * TC_M, n0 = blockIdx.y * TC_N;
  const uint32_t btma = smem_u32(&bar_tma), bmma = smem_u32(&bar_mma);

  if (t == 0) {
    s_fail = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(btma) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bmma) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  // this thread's row of A: mode k, real (c = 0) or imaginary (c = 1) part
  const int r = m0 + t, k = r >> 1, c = r & 1;
  const bool rowok = k < Nk && !(c == 1 && jb.x_real);
  const double2* xr = jb.X + (long long)(k < Nk ? k : 0) * N;
  double amax = 0.0;
  if (rowok)
    for (int m = 0; m < N; ++m) {
      const double2 v = xr[m];
      amax = fmax(amax, fabs(c ? v.y : v.x));
    }
  int e = 0;
  if (amax > 0.0) frexp(amax, &e);

  bool seen[TC_SLICES];
  for (int p = 0; p < TC_SLICES; ++p) seen[p] = false;
  for (int ch = 0; ch < nchunks; ++ch) {
    const uint32_t phase = (uint32_t)(ch & 1);
    if (t == 0) {
      const unsigned char* src = static_cast<const unsigned char*>(jb.bslices) +
                                 ((long long)blockIdx.y * nchunks + ch) * TC_B_CHUNK_BYTES;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(btma),
                   "r"(TC_B_CHUNK_BYTES)
                   : "memory");
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
              "r"(smem_u32(sB)),
          "l"(src), "r"(TC_B_CHUNK_BYTES), "r"(btma)
          : "memory");
    }
    // the 32 values of this chunk, cut into slices (integer arithmetic on
    // the FP64 bits: the 56 bits below 2^e, 7 per slice), 8 per 16-byte row
    for (int kb = 0; kb < 4; ++kb) {
      unsigned short sl[TC_SLICES][8];
      for (int i = 0; i < 8; ++i) {
        const int m = ch * TC_KC + kb * 8 + i;
        unsigned long long u = 0;
        bool neg = false;
        if (rowok && m < N) u = fixed56(c ? xr[m].y : xr[m].x, e, &neg);
        for (int p = 0; p < TC_SLICES; ++p)
          sl[p][i] = bf16_int((unsigned)((u >> (49 - 7 * p)) & 127u), neg);
      }
      const int off = tc_off(t, kb * 8);
      for (int p = 0; p < TC_SLICES; ++p) {
        uint4 w;
        w.x = (uint32_t)sl[p][0] | ((uint32_t)sl[p][1] << 16);
        w.y = (uint32_t)sl[p][2] | ((uint32_t)sl[p][3] << 16);
        w.z = (uint32_t)sl[p][4] | ((uint32_t)sl[p][5] << 16);
        w.w = (uint32_t)sl[p][6] | ((uint32_t)sl[p][7] << 16);
        *reinterpret_cast<uint4*>(sA + p * TC_A_SLICE_BYTES + off) = w;
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (t == 0) {
      if (!mbar_wait(btma, phase)) s_fail = 1;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (!s_fail) {
        for (int p = 0; p < TC_SLICES; ++p)
          for (int q = 0; p + q < TC_SLICES; ++q) {
            const int lv = p + q;
            for (int ks = 0; ks < TC_KC / 16; ++ks) {
              const uint64_t ad = sdesc(smem_u32(sA + p * TC_A_SLICE_BYTES + ks * 256), 128, 512);
              const uint64_t bd = sdesc(smem_u32(sB + q * TC_B_SLICE_BYTES + ks * 256), 128, 512);
              const uint32_t acc = seen[lv] ? 1u : 0u;
              asm volatile(
                  "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                  " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
                      tmem + (uint32_t)(lv * TC_N)),
                  "l"(ad), "l"(bd), "r"(TC_IDESC), "r"(acc)
                  : "memory");
              seen[lv] = true;
            }
          }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       bmma)
                   : "memory");
    }
    __syncthreads();
    // the MMAs of this chunk have read sA / sB (and written TMEM) before the
    // next chunk overwrites them
    if (!mbar_wait(bmma, phase)) s_fail = 1;
    __syncthreads();
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const bool failed = s_fail != 0;
  if (failed) {
    // give MMAs that may still be in flight one more bounded wait before
    // their tensor memory is read and freed
    mbar_wait(bmma, (uint32_t)((nchunks - 1) & 1));
    if (t == 0) atomicExch(err, 1);
  }

  // epilogue: warp w holds TMEM lanes 32w .. 32w + 31 = rows m0 + 32 w + lane;
  // level lv (weight 2^(-7 (lv + 2)) of the scales) enters the integer sum
  // with weight 2^(38 - 7 lv), i.e. in units of 2^-52 of the scales (lv > 5:
  // shifted right, dropping less than a unit each)
  const double rs = ldexp(1.0, e - 52);
  for (int cg = 0; cg < TC_N / 16; ++cg) {
    long long acc[16];
    for (int j = 0; j < 16; ++j) acc[j] = 0;
    for (int lv = TC_SLICES - 1; lv >= 0; --lv) {
      uint32_t v[16];
      const uint32_t ta = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(lv * TC_N + cg * 16);
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
        const long long d = (long long)__float2int_rz(__uint_as_float(v[j]));   // exact: < 2^24
        acc[j] += lv <= 5 ? (d << (38 - 7 * lv)) : (d >> (7 * lv - 38));
      }
    }
    for (int j = 0; j < 16; ++j) {
      const int n = n0 + cg * 16 + j;
      double val = failed ? NAN : __ll2double_rn(acc[j]) * rs * (n < N ? jb.bscale[n] : 0.0);
      const double im = __shfl_down_sync(0xffffffffu, val, 1);
      if (c == 0 && k < Nk && n < N) {
        double2* yp = jb.Y + (long long)k * N + n;
        if (jb.zero_tau && n >= N - 2) {
          if (!jb.accumulate) *yp = make_double2(0.0, 0.0);
        } else {
          const double2 f = kfactor_eval(jb.f, kx ? kx[k] : 0.0);
          double2 out = make_double2(f.x * val - f.y * im, f.x * im + f.y * val);
          if (jb.accumulate) out = cadd(*yp, out);
          *yp = out;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TC_TMEM_COLS)
                 : "memory");
}

}  // namespace

TcCache::~TcCache() {
  for (void* p : owned) cudaFree(p);
}

const TcOperator* TcCache::get(const Ctx& c, const double* Z) {
  auto it = ops.find(Z);
  if (it != ops.end()) return &it->second;
  auto reg = registered.find(Z);
  if (reg == registered.end()) return nullptr;
  TcOperator op;
  op.rows = reg->second;
  op.K = K;
  op.ntiles = ceil_div(op.rows, TC_N);
  op.nchunks = ceil_div(K, TC_KC);
  const size_t bytes = (size_t)op.ntiles * op.nchunks * TC_B_CHUNK_BYTES;
  SMC_CUDA(cudaMalloc(&op.slices, bytes));
  owned.push_back(op.slices);
  SMC_CUDA(cudaMalloc((void**)&op.scale, sizeof(double) * op.ntiles * TC_N));
  owned.push_back(op.scale);
  SMC_CUDA(cudaMemsetAsync(op.slices, 0, bytes, c.s));
  SMC_CUDA(cudaMemsetAsync(op.scale, 0, sizeof(double) * op.ntiles * TC_N, c.s));
  smc_tc_pack_kernel<<<ceil_div(op.rows, 4), 128, 0, c.s>>>(
      Z, op.rows, K, op.nchunks, static_cast<unsigned char*>(op.slices), op.scale);
  SMC_LAUNCH_CHECK(c);
  return &(ops[Z] = op);
}

bool tc_zmat_apply(const Ctx& c, TcCache& cache, const ZJob* jobs, int njobs, int Nk, int N,
                   const double* kx) {
  if (njobs < 1 || njobs > 4 || N > TC_KMAX || N != cache.K || !cache.err) return false;
  for (int i = 0; i < njobs; ++i) {
    auto it = cache.registered.find(jobs[i].Z);
    if (jobs[i].zstride != 0 || it == cache.registered.end() || it->second != N) return false;
  }
  TcJobs4 js;
  for (int i = 0; i < njobs; ++i) {
    const TcOperator* op = cache.get(c, jobs[i].Z);
    js.j[i].X = jobs[i].X;
    js.j[i].Y = jobs[i].Y;
    js.j[i].bslices = op->slices;
    js.j[i].bscale = op->scale;
    js.j[i].f = jobs[i].f;
    js.j[i].accumulate = jobs[i].accumulate;
    js.j[i].x_real = jobs[i].x_real;
    js.j[i].zero_tau = jobs[i].zero_tau;
  }
  static bool attr = false;
  if (!attr) {
    SMC_CUDA(cudaFuncSetAttribute((const void*)smc_tc_zmat_kernel,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
    attr = true;
  }
  dim3 grd(ceil_div(2LL * Nk, TC_M), ceil_div(N, TC_N), njobs);
  smc_tc_zmat_kernel<<<grd, TC_THREADS, TC_SMEM, c.s>>>(js, Nk, N, ceil_div(N, TC_KC), kx,
                                                        cache.err);
  SMC_LAUNCH_CHECK(c);
  return true;
}

}  // namespace smc
