// smc_grid_noalloc: the Fourier x Chebyshev synthesis of smc_transform
// (SMC_GRID / SMC_SYNTH_PAD) for callers that cannot allocate device memory.
//
// Who needs it: code that owns all device memory through its own fixed arena
// (a host framework whose allocator forbids foreign cudaMalloc calls), and
// time loops that must never stall the device -- cudaMalloc/cudaFree can
// synchronise the whole device, which a caller interleaving its own kernels
// on other streams cannot afford.  Such callers cannot create a model handle
// (smc_create allocates its buffers), but they can still turn spectral
// coefficients they hold into grid values with this entry point.
//
// The synthesis runs in two kernels (a z-contraction with the Chebyshev
// Vandermonde, then a real inverse DFT along x), and the intermediate
// "values per x-mode" array between them lives in the fixed device array
// g_noalloc_modes below instead of an allocated buffer.  The array is part of
// the library image: every GPU that loads the library holds it (8 MiB) until
// the process exits.  Every call overwrites each entry it later reads, so
// nothing has to start at zero; but all calls share the one array, so calls
// that overlap on the GPU (concurrent streams, or host threads issuing to
// different streams without ordering) race and corrupt each other's results.
#include <algorithm>
#include <mutex>

#include "../../include/specmc_gb300.h"
#include "smc_internal.cuh"

namespace smc {

void set_last_error(const char* msg);   // smc_runtime.cu

// largest Nk * Nz the no-allocation synthesis accepts (complex entries)
static constexpr long long NOALLOC_MAX_MODES = SMC_NOALLOC_MAX_MODES;
static __device__ __align__(256) double2 g_noalloc_modes[NOALLOC_MAX_MODES];

// device address of g_noalloc_modes per device, looked up once per device
static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[64] = {nullptr};

// X[k][j] = sum_n T_n(2 z_j - 1) c[k][n], z_j the ascending CGL nodes:
// T_n(-cos(pi j/(N-1))) = (-1)^n cos(pi n j/(N-1)), evaluated with an exact
// angle reduction
__global__ void smc_noalloc_zsynth_kernel(const double2* __restrict__ c, double2* __restrict__ X,
                                          int Nk, int N) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  const long long period = 2LL * (N - 1);
  // rows k stride over gridDim.y (at most 65535), so every Nk is covered
  for (int k = blockIdx.y; k < Nk; k += gridDim.y) {
    const double2* ck = c + (long long)k * N;
    double sr = 0.0, si = 0.0;
    for (int n = 0; n < N; ++n) {
      double t = cospi((double)(((long long)n * j) % period) / (double)(N - 1));
      if (n & 1) t = -t;
      sr += t * ck[n].x;
      si += t * ck[n].y;
    }
    X[(long long)k * N + j] = make_double2(sr, si);
  }
}

// g[i][j] = Re X[0][j] + sum_{k>=1} w_k Re(X[k][j] e^{2 pi i k i / Ng}),
// w_k = 2 except the Nyquist mode 2k = Ng (weight 1)
__global__ void smc_noalloc_xsynth_kernel(const double2* __restrict__ X, double* __restrict__ g,
                                          int Nk, int N, int Ng) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  // grid rows i stride over gridDim.y (at most 65535), so every Ng is covered
  for (int i = blockIdx.y; i < Ng; i += gridDim.y) {
    double acc = X[j].x;
    for (int k = 1; k < Nk; ++k) {
      double s, c;
      sincospi(2.0 * (double)(((long long)k * i) % Ng) / (double)Ng, &s, &c);
      double2 x = X[(long long)k * N + j];
      double v = x.x * c - x.y * s;
      acc += (2 * k == Ng) ? v : 2.0 * v;
    }
    g[(long long)i * N + j] = acc;
  }
}

}  // namespace smc

extern "C" int smc_grid_noalloc(const double* that_dev, double* grid_dev, int Nx, int Nz,
                                int padded, void* stream) {
  using namespace smc;
  try {
    if (!that_dev || !grid_dev) throw std::runtime_error("smc_grid_noalloc: null pointer");
    if (Nx < 4 || Nz < 4 || (Nx % 2))
      throw std::runtime_error("smc_grid_noalloc: Nx must be even and >= 4, Nz >= 4");
    const int Nk = Nx / 2 + 1;
    const long long modes = (long long)Nk * Nz;
    if (modes > NOALLOC_MAX_MODES)
      throw std::runtime_error("smc_grid_noalloc: (Nx/2+1)*Nz = " + std::to_string(modes) +
                               " exceeds the fixed scratch of " +
                               std::to_string(NOALLOC_MAX_MODES) + " complex entries");
    int dev = 0;
    SMC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) throw std::runtime_error("smc_grid_noalloc: device ordinal >= 64");
    void* scratch = nullptr;
    {
      // set-up once per device, with that device current: the host-side
      // name of a __device__ array is not a device address
      std::lock_guard<std::mutex> lk(g_noalloc_mu);
      if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        SMC_CUDA(cudaGetSymbolAddress(&p, g_noalloc_modes));
        g_noalloc_addr[dev] = p;
      }
      scratch = g_noalloc_addr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double2* X = static_cast<double2*>(scratch);
    const int Ng = padded ? 2 * Nx : Nx;
    // gridDim.y is capped at 65535; the kernels stride their rows over it
    smc_noalloc_zsynth_kernel<<<dim3(ceil_div(Nz, 128), std::min(Nk, 65535)), 128, 0, s>>>(
        reinterpret_cast<const double2*>(that_dev), X, Nk, Nz);
    SMC_CUDA(cudaGetLastError());
    smc_noalloc_xsynth_kernel<<<dim3(ceil_div(Nz, 128), std::min(Ng, 65535)), 128, 0, s>>>(X, grid_dev, Nk, Nz, Ng);
    SMC_CUDA(cudaGetLastError());
    return 0;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return -1;
  }
}
