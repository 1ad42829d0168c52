// Allocation-free batched gradient (gnuts_log_prob_grad_noalloc).
//
// For callers that cannot allocate device memory (a memory pool or arena
// that owns every device allocation, a callback running inside another
// library, an allocator-free real-time loop) but can hand over device
// buffers for inputs and outputs.  The batched logistic / horseshoe gradient
// normally allocates its scratch per call (coefficient rows, row-split
// partial sums); here that scratch is one file-scope static device array of
// GNUTS_NOALLOC_SCRATCH_BYTES, present on every GPU that loads the library
// until the process exits.  Nothing in this file calls cudaMalloc, cudaFree
// or an allocating library routine.
//
// The array's name is a host-side stand-in in host code, not a device
// address: its device address is looked up with cudaGetSymbolAddress once
// per device (first call on that device, with the device current) and passed
// to the kernels.  Every call overwrites the whole part of the scratch it
// reads (coefficients, every split's partials, the reduced sums), so nothing
// needs clearing between calls; calls that overlap on the GPU race on it.
#include <cuda_runtime.h>
#include <algorithm>
#include <mutex>
#include <string>
#include "internal.h"
#include "batched.cuh"

namespace gnuts {
namespace {

constexpr size_t kScratchDoubles = GNUTS_NOALLOC_SCRATCH_BYTES / sizeof(double);
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_addr[kMaxDevices] = {};

__global__ void k_na_stage(GradOut G, DevModel M, int n, const double* q) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  stage_request(G, M, warp, q + (size_t)warp * M.D, lane);
}

__global__ void k_na_finish(GradOut G, DevModel M, int n, const double* q, int jac, double* lp, double* g) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  double v = reduce_gradient(G, M, warp, q + (size_t)warp * M.D, g + (size_t)warp * M.D, lane);
  if (!jac && M.kind == MK_HORSESHOE) {
    // reduce_gradient includes the Jacobian of the positive transforms
    const int K = M.K;
    const double* qq = q + (size_t)warp * M.D;
    double* gg = g + (size_t)warp * M.D;
    double jl = 0;
    for (int d = lane; d < K; d += 32) {
      jl += qq[K + 2 + d];
      gg[K + 2 + d] -= 1.0;
    }
    jl = wsum(jl);
    v -= jl + qq[K + 1] + qq[2 * K + 2];
    __syncwarp();
    if (lane == 0) {
      gg[K + 1] -= 1.0;
      gg[2 * K + 2] -= 1.0;
    }
  }
  if (lane == 0) lp[warp] = v;
}

}  // namespace

int noalloc_log_prob_grad(const Model& m, int n, const double* q, int jac, double* lp, double* g, std::string& err) {
  const DevModel& M = m.dev;
  if (!batched_supported(M)) {
    err = "gnuts_log_prob_grad_noalloc covers the batched models (logistic, horseshoe); use gnuts_log_prob_grad";
    return GNUTS_ERR_ARGUMENT;
  }
  if (n < 1 || n > GNUTS_NOALLOC_MAX_POINTS) {
    err = "gnuts_log_prob_grad_noalloc: n = " + std::to_string(n) + " is outside 1.." +
          std::to_string(GNUTS_NOALLOC_MAX_POINTS) + " (GNUTS_NOALLOC_MAX_POINTS)";
    return GNUTS_ERR_ARGUMENT;
  }
  if (M.K + 1 > GNUTS_NOALLOC_MAX_COEF) {
    err = "gnuts_log_prob_grad_noalloc: " + std::to_string(M.K) + " predictors exceed GNUTS_NOALLOC_MAX_COEF - 1 = " +
          std::to_string(GNUTS_NOALLOC_MAX_COEF - 1);
    return GNUTS_ERR_ARGUMENT;
  }
  if (!q || !lp || !g) {
    err = "gnuts_log_prob_grad_noalloc: null device buffer";
    return GNUTS_ERR_ARGUMENT;
  }
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    err = std::string("gnuts_log_prob_grad_noalloc: no usable current device: ") + cudaGetErrorString(e);
    return GNUTS_ERR_CUDA;
  }
  if (m.device != dev || !M.X) {
    err = "gnuts_log_prob_grad_noalloc: the model's data is not on the current device yet; make one allocating "
          "device call on this model first (for example gnuts_log_prob_grad), which uploads it";
    return GNUTS_ERR_ARGUMENT;
  }
  double* scratch;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        err = std::string("gnuts_log_prob_grad_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
        return GNUTS_ERR_CUDA;
      }
      g_scratch_addr[dev] = (double*)p;
    }
    scratch = g_scratch_addr[dev];
  }
  // split the rows like the allocating path, at most GNUTS_NOALLOC_MAX_SPLITS splits
  GradOut G{};
  G.kind = M.kind;
  G.prec = GNUTS_PRECISION_FP64;
  G.C = n;
  G.C_total = n;
  G.K = M.K;
  const int ctiles = (n + GLM_CT - 1) / GLM_CT;
  int S = std::max(1, (152 * 4 + ctiles - 1) / ctiles);
  S = std::min(S, std::max(1, M.N / 256));
  int rps = (M.N + S - 1) / S;
  rps = (rps + GLM_RB - 1) / GLM_RB * GLM_RB;
  S = (M.N + rps - 1) / rps;
  if (S > GNUTS_NOALLOC_MAX_SPLITS) {
    rps = (M.N + GNUTS_NOALLOC_MAX_SPLITS - 1) / GNUTS_NOALLOC_MAX_SPLITS;
    rps = (rps + GLM_RB - 1) / GLM_RB * GLM_RB;
    S = (M.N + rps - 1) / rps;
  }
  G.S = S;
  G.rows_per_split = rps;
  const size_t K1 = (size_t)M.K + 1;
  G.part_g = scratch;                                   // S x n x (K+1)
  G.part_lp = G.part_g + (size_t)S * n * K1;            // S x n
  G.coef64 = scratch + (size_t)GNUTS_NOALLOC_MAX_SPLITS * GNUTS_NOALLOC_MAX_POINTS * (GNUTS_NOALLOC_MAX_COEF + 1);
  (void)cudaGetLastError();
  const int blocks = (n * 32 + 127) / 128;
  k_na_stage<<<blocks, 128>>>(G, M, n, q);
  dim3 grid((unsigned)ctiles, (unsigned)S);
  if (M.K <= GLM_KC) k_glm_simt<double, 1><<<grid, GLM_THREADS>>>(G, M);
  else k_glm_simt<double, 8><<<grid, GLM_THREADS>>>(G, M);
  k_na_finish<<<blocks, 128>>>(G, M, n, q, jac, lp, g);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  if (e != cudaSuccess) {
    err = std::string("gnuts_log_prob_grad_noalloc: CUDA error: ") + cudaGetErrorString(e);
    return GNUTS_ERR_CUDA;
  }
  return GNUTS_OK;
}

}  // namespace gnuts
