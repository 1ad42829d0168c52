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
// Execution of the SIMT kernels (training, the public forward / log-density
// entry points): one warp per point, up to 4 points per CTA.  The CTA streams one
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
  long wt_off[FLOW_MAX_L];          // layer blocks of w16t (tensor-core layout)
  int stage_max_tc;                 // largest tensor-core stage in BF16 elements
  const int* idx;
  const float* theta;
  const __nv_bfloat16* w16;
  const __nv_bfloat16* w16t;
};

// Tensor-core layout of layer l's weights (w16t), four zero-padded row-major
// BF16 matrices, each the A operand of one m16n8k16 contraction whose B
// operand holds one point per column:
//   forward stage  [F1 = W1^T  H  x kb  | F2 = W2^T  ma x H ]
//   adjoint stage  [A3 = W2    H  x ma  | A4 = W1    kb x H ]
// kb = n_b rounded up to 16, ma = 2 n_a rounded up to 16; every row is
// stored with 8 extra elements so that the eight rows one fragment load
// touches fall in distinct shared-memory banks.  Padding is zero.
__host__ __device__ inline int tc_pad16(int n) { return (n + 15) & ~15; }
__host__ __device__ inline long tc_fwd_elems(int H, int nb, int na) {
  return (long)H * (tc_pad16(nb) + 8) + (long)tc_pad16(2 * na) * (H + 8);
}
__host__ __device__ inline long tc_adj_elems(int H, int nb, int na) {
  return (long)H * (tc_pad16(2 * na) + 8) + (long)tc_pad16(nb) * (H + 8);
}

// Shared memory of the tensor-core gradient pass for T points (offsets in
// floats from the start of the pass's area, after the index table and the
// two weight-stage buffers):
//   sig    [d] FP64 exp(rho), computed once per launch
//   region [T][pr] FP32 per point: x, gx (FP64), y, ybar, r (GEMM2 output),
//          tape h [L][H], s [L][namax], u_a [L][namax];
//          pr = 4 (mod 8), so a warp's epilogue stores (rows m0..m0+7 of
//          four points) hit distinct banks
//   four B-operand arrays in BF16, each [3 parts][T][stride] with
//          stride = 8 (mod 16) elements, so the 32-bit fragment loads of a
//          warp (eight points x four k pairs) hit distinct banks:
//          ub (n_b inputs, kbmax + 8), rb (output adjoints, mamax + 8),
//          pb (hidden adjoints, H + 8), hb (hidden activations, H + 8)
struct FlowTcLayout {
  int o_x, o_gx, o_y, o_yb, o_r, o_h, o_s, o_ua;  // within a point region
  int h_stride, s_stride, pr;
  int o_sig, o_regions;                          // floats from the area start
  int o_ub, o_rb, o_pb, o_hb;                    // BF16 elements from the area start
  int ub_stride, rb_stride, pb_stride;           // point strides (hb: pb_stride)
  int T;
  size_t bytes;                                  // area size
};

__host__ __device__ inline FlowTcLayout flow_tc_layout(const FlowDev& F, int T) {
  FlowTcLayout t{};
  int kbmax = 16, mamax = 16, namax = 1;
  for (int l = 0; l < F.L; ++l) {
    kbmax = tc_pad16(F.nb[l]) > kbmax ? tc_pad16(F.nb[l]) : kbmax;
    mamax = tc_pad16(2 * F.na[l]) > mamax ? tc_pad16(2 * F.na[l]) : mamax;
    namax = F.na[l] > namax ? F.na[l] : namax;
  }
  const int d4 = (F.d + 3) & ~3;
  int o = 0;
  t.o_x = o;  o += 2 * F.d;
  t.o_gx = o; o += 2 * F.d;
  t.o_y = o;  o += d4;
  t.o_yb = o; o += d4;
  t.o_r = o;  o += mamax;
  t.h_stride = F.H;
  t.o_h = o;  o += F.L * t.h_stride;
  t.s_stride = (namax + 3) & ~3;
  t.o_s = o;  o += F.L * t.s_stride;
  t.o_ua = o; o += F.L * t.s_stride;
  o = (o + 3) & ~3;
  if (o % 8 != 4) o += 4;
  t.pr = o;
  t.T = T;
  t.o_sig = 0;
  t.o_regions = (2 * F.d + 3) & ~3;
  const int fl = t.o_regions + T * t.pr;  // floats so far
  t.ub_stride = kbmax + 8;
  t.rb_stride = mamax + 8;
  t.pb_stride = F.H + 8;
  int e = 2 * fl;                          // BF16 elements so far
  t.o_ub = e; e += 3 * T * t.ub_stride;
  t.o_rb = e; e += 3 * T * t.rb_stride;
  t.o_pb = e; e += 3 * T * t.pb_stride;
  t.o_hb = e; e += 3 * T * t.pb_stride;
  t.bytes = (size_t)e * 2;
  t.bytes = (t.bytes + 15) & ~(size_t)15;
  return t;
}

// 16-byte asynchronous global -> shared copies (weight staging)
__device__ __forceinline__ void fl_cp16(void* s, const void* g) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(s)), "l"(g)
               : "memory");
}
__device__ __forceinline__ void fl_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void fl_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

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

// shared memory of the tensor-core pass for T points: index table, two
// weight-stage buffers, the pass's area
__host__ __device__ inline size_t flow_tc_bytes(const FlowDev& F, int T) {
  return flow_align16(sizeof(int) * (size_t)F.L * F.d) + 2 * flow_align16(2 * (size_t)F.stage_max_tc) +
         flow_tc_layout(F, T).bytes;
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

// flow_tc_kind.cu (one object per model kind): the fused flow sampler and
// the standalone gradient pass on the tensor cores; FLOW_TC_W warps per CTA
// (each contraction has at most 8 m-tiles, one per warp)
constexpr int FLOW_TC_W = 8;
struct Params;
struct Bufs;
template <int KIND>
cudaError_t flow_tc_fused_launch_k(const FlowDev& F, const Params& P, const Bufs& B, const DevModel& M, int T,
                                   size_t flow_bytes, int blocks, size_t smem);
template <int KIND>
cudaError_t flow_tc_grad_launch_k(const FlowDev& F, const DevModel& M, int n, int T, const double* z, double* lp,
                                  double* g, size_t smem);

}  // namespace gnuts
