// Affine-coupling flow on the device: the learned preconditioner that NUTS
// samples through.  No counterpart in the reference (CmdStan samples the
// model's own unconstrained space); the sampler it wraps is the one behind
// stan::services::sample::hmc_nuts_diag_e_adapt (src/cmdstan/command.hpp:
// 673-688).
//
// Map z -> x (RealNVP coupling layers, Dinh et al. 2017):
//   u_0 = z;  u_{l+1} = f_l(u_l);  x = mu + exp(rho) .* u_L
//   f_l keeps the conditioner set b_l and transforms the set a_l:
//     pre = W1^T u_b + b1 (H hidden units), h = tanh(pre),
//     r = W2^T h + b2 (2 n_a outputs), s = c tanh(r_s / c), t = r_t,
//     y_a = u_a .* exp(s) + t,   y_b = u_b.
//   Index i is in b_l when bit (l mod B) of i equals (l div B) mod 2,
//   B = ceil(log2 d): any two dimensions are split apart by some layer.
//   log|det dx/dz| = sum_l sum s_l + sum rho.
// The sampler's target in z is lp_x(T(z)) + log|det|; its gradient is the
// adjoint sweep J^T grad_x plus the log-determinant's own gradient.
//
// Parameters live in one FP32 vector theta (per layer W1 [n_b][H], b1 [H],
// W2 [H][2 n_a], b2 [2 n_a]; then mu [d], rho [d]); the weight matrices are
// also kept in BF16 (the sampler and the training forward use those; Adam
// updates the FP32 master) in a per-layer block [W2 | W1 | W2^T] so that a
// forward stage streams [W2 | W1] and an adjoint stage [W1 | W2^T], each one
// contiguous range.
//
// Execution: one warp per point, FLOW_T points per CTA.  The CTA streams one
// layer's BF16 weights at a time into shared memory with cp.async (double
// buffered: the next stage's copy is in flight while this stage computes),
// so every warp of the CTA reads them on chip.  Lane l owns hidden units
// HPL*l .. HPL*l+HPL-1 (HPL = H/32); FP32 arithmetic, FP32 accumulation; the
// model's log density and gradient at x stay FP64.
#pragma once
#include <cuda_bf16.h>
#include "device_models.cuh"
#include "philox.cuh"

namespace gnuts {

constexpr int FLOW_MAX_L = 16;
constexpr int FLOW_MAX_D = 128;  // n_a <= 64, so 2 n_a outputs fit two 64-column passes

struct FlowDev {
  int d, L, H;
  float clamp;
  int nb[FLOW_MAX_L], na[FLOW_MAX_L];
  int idx_off[FLOW_MAX_L];          // into idx: layer l's b list (n_b) then a list (n_a)
  long th_off[FLOW_MAX_L + 1];      // layer blocks of theta; th_off[L] = offset of mu
  long th_rho, n_params;
  long w_off[FLOW_MAX_L];           // layer blocks of w16 (BF16 elements)
  int stage_max;                    // largest stage in BF16 elements
  const int* idx;
  const float* theta;
  const __nv_bfloat16* w16;
};

// points (warps) per CTA and shared-memory plan
struct FlowPlan {
  int T;
  size_t idx_bytes, wbuf_bytes, warp_bytes, total;
  int namax;
};

__host__ __device__ inline size_t flow_align16(size_t b) { return (b + 15) & ~(size_t)15; }

__host__ __device__ inline void flow_warp_layout(const FlowDev& F, int namax, int* tape_floats) {
  int t = 0;
  for (int l = 0; l < F.L; ++l) t += F.d + F.H + F.na[l];
  *tape_floats = t + F.d;  // + u_L
}

// bytes of one warp's region: x, gx (FP64); y, ybar, sc (2 n_a max or H),
// pb (H), tape (FP32)
__host__ __device__ inline size_t flow_warp_bytes(const FlowDev& F, int namax) {
  int tape;
  flow_warp_layout(F, namax, &tape);
  const int scn = 2 * namax > F.H ? 2 * namax : F.H;
  return flow_align16(16 * (size_t)F.d + 4 * ((size_t)2 * F.d + scn + F.H + tape));
}

inline FlowPlan flow_plan(const FlowDev& F, size_t smem_limit) {
  FlowPlan p{};
  p.namax = 0;
  for (int l = 0; l < F.L; ++l) p.namax = F.na[l] > p.namax ? F.na[l] : p.namax;
  p.idx_bytes = flow_align16(sizeof(int) * (size_t)F.L * F.d);
  p.wbuf_bytes = flow_align16(2 * (size_t)F.stage_max);
  p.warp_bytes = flow_warp_bytes(F, p.namax);
  for (int T = 4; T >= 1; T >>= 1) {
    p.T = T;
    p.total = p.idx_bytes + 2 * p.wbuf_bytes + T * p.warp_bytes;
    if (p.total <= smem_limit) return p;
  }
  p.T = 0;
  return p;
}

}  // namespace gnuts
