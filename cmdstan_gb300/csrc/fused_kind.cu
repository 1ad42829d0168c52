// Fused-mode kernel: each warp runs one chain's NUTS state machine and
// evaluates its model's gradient itself (the log_prob_grad contract of
// stan::model, src/cmdstan/command_helper.hpp:589-593), up to
// P.grad_budget gradients per launch.
//
// This file is compiled once per model kind (-DGNUTS_KIND=k): each object
// carries one instantiation with only its own model's gradient code, so the
// state machine and that gradient share the register file without the
// spills a kernel holding every model's code has; the objects also compile
// in parallel.  fused.cu dispatches on the model's kind.
#include <cuda_runtime.h>
#include "internal.h"
#include "nuts_device.cuh"

#ifndef GNUTS_KIND
#error "compile with -DGNUTS_KIND=<model kind>"
#endif

namespace gnuts {

template <int KIND>
__global__ void __launch_bounds__(128) k_fused(Params P, Bufs B, DevModel M, ReplayBufs RB) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= P.C) return;
  Scal s = B.sc[warp];
  if (s.phase >= PH_DONE) return;
  const DevModel& Mc = chain_model(M, warp, P.C);
  Chain ch(P, B, Mc, s, warp, lane);
  if (RB.chain_ids) ch.chain_id = RB.chain_ids[warp];
  extern __shared__ double gn_cache[];
  if (P.cache) ch.cache_attach(gn_cache + (size_t)(threadIdx.x >> 5) * P.cache_stride);
  for (int b = 0; b < P.grad_budget; ++b) {
    double lp = warp_lpg_k<KIND>(Mc, ch.Wq, ch.Wg, 1, lane);
    __syncwarp();
    s.W_lp = lp;
    if (!ch.advance()) break;
  }
  if (P.cache) ch.cache_detach();
  __syncwarp();
  if (lane == 0) B.sc[warp] = s;
}

template <int KIND>
cudaError_t fused_set_smem_k(int bytes) {
  return cudaFuncSetAttribute(k_fused<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <int KIND>
cudaError_t fused_launch_k(int blocks, int threads, size_t smem, const Params& P, const Bufs& B, const DevModel& M,
                           const ReplayBufs& RB) {
  k_fused<KIND><<<blocks, threads, smem>>>(P, B, M, RB);
  return cudaGetLastError();
}

template cudaError_t fused_set_smem_k<GNUTS_KIND>(int);
template cudaError_t fused_launch_k<GNUTS_KIND>(int, int, size_t, const Params&, const Bufs&, const DevModel&,
                                                const ReplayBufs&);

}  // namespace gnuts
