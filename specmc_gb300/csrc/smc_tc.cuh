// Tensor-core (tcgen05) z-contractions with FP64 accuracy (smc_tc.cu).
#pragma once
#include <memory>
#include <unordered_map>
#include <vector>

#include "smc_internal.cuh"

namespace smc {

constexpr int TC_SLICES = 8;            // 7-bit slices: 56 bits of each operand
constexpr int TC_M = 128;               // A rows per CTA (= TMEM lanes)
constexpr int TC_N = 32;                // B rows (outputs) per CTA
constexpr int TC_KC = 32;               // K per chunk (two MMA k-steps of 16)
constexpr int TC_A_SLICE_BYTES = TC_M * TC_KC * 2;
constexpr int TC_B_SLICE_BYTES = TC_N * TC_KC * 2;
constexpr int TC_B_CHUNK_BYTES = TC_SLICES * TC_B_SLICE_BYTES;
constexpr int TC_KMAX = 128;            // exactness bound of the FP32 accumulation

// An operator Z (rows x K, FP64, row-major) split for the tensor cores:
// per row q an exponent f_q with max_m |Z[q][m]| < 2^f_q, and TC_SLICES
// bf16 slices of 7 bits each of Z[q][m] 2^-f_q, stored tile by tile in the
// exact shared-memory image the MMA reads (32-row tiles, 32-column K chunks,
// 8 x 16-byte core matrices), so a K chunk of a tile is one bulk copy.
struct TcOperator {
  int rows = 0, K = 0, ntiles = 0, nchunks = 0;
  void* slices = nullptr;      // bf16, ntiles * nchunks * TC_B_CHUNK_BYTES
  double* scale = nullptr;     // 2^f_q, rows (padded to ntiles * TC_N)
};

// The tensor-core operators of a model: registered once per immutable
// matrix (the Chebyshev V, V^-1, D, D^2 ... of the handle), split on first
// use.  Jobs whose Z is not registered (or per-k operators) use the FP64
// SIMT contraction.
struct TcCache {
  std::unordered_map<const double*, TcOperator> ops;
  std::unordered_map<const double*, int> registered;   // Z -> rows (= N)
  std::vector<void*> owned;
  int K = 0;                   // the contraction length (Nz) of every registered operator
  int* err = nullptr;          // device flag: a tensor-core CTA timed out waiting (results NaN)
  ~TcCache();
  void add(const double* Z, int rows) { registered[Z] = rows; }
  const TcOperator* get(const Ctx& c, const double* Z);
};

// Y_b[k][n] (=|+=) f_b(k) sum_m Z_b[n][m] X_b[k][m] for jobs whose Z is in
// the cache (zstride 0, N <= TC_KMAX): on the tensor cores, FP64 accuracy
// (Ozaki splitting into bf16 slices, exact FP32 accumulation in TMEM).
// Returns false (nothing launched) when some job cannot take this path.
bool tc_zmat_apply(const Ctx& c, TcCache& cache, const ZJob* jobs, int njobs, int Nk, int N,
                   const double* kx);

}  // namespace smc
