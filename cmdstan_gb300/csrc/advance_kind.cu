// Round-mode state-machine step: every live chain sums its gradient from
// the batched kernel's partials (reduce_gradient), advances its NUTS state
// machine to the next gradient request (Chain::advance) and stages the
// coefficient row of that request (stage_request).
//
// This file is compiled once per (metric, team width) pair
// (-DGNUTS_MET=m -DGNUTS_TW=w): each object holds one instantiation, so they
// build in parallel, and the diag_e kernel carries no dense-metric code.
#include <cuda_runtime.h>
#include "internal.h"
#include "advance.h"

#if !defined(GNUTS_MET) || !defined(GNUTS_TW)
#error "compile with -DGNUTS_MET=<metric> -DGNUTS_TW=<team width>"
#endif

namespace gnuts {

// TW = 32: one warp per chain, four chains per CTA.  TW > 32: one chain per
// CTA of TW threads (wide chains).
template <int MET, int TW>
__global__ void __launch_bounds__(TW == 32 ? 128 : TW) k_advance(Params P, Bufs B, DevModel M, GradOut G) {
  const int chain = TW == 32 ? (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) : (int)blockIdx.x;
  const int lane = TW == 32 ? (int)(threadIdx.x & 31) : (int)threadIdx.x;
  if (chain >= P.C) return;
  Scal s = B.sc[chain];
  if (s.phase >= PH_DONE) return;
  Chain<MET, TW> ch(P, B, M, s, chain, lane);
  extern __shared__ double gn_cache[];
  if (P.cache) ch.cache_attach(gn_cache + (size_t)(threadIdx.x >> 5) * P.cache_stride);
  // gather this chain's gradient from the batched kernel's partial sums
  s.W_lp = reduce_gradient<TW>(G, M, chain, ch.Wq, ch.Wg, lane);
  tsync<TW>();
  bool more = ch.advance();
  if (more) stage_request<TW>(G, M, chain, ch.Wq, lane);
  if (P.cache) ch.cache_detach();
  tsync<TW>();
  if (lane == 0) B.sc[chain] = s;
}

template <int MET, int TW>
cudaError_t advance_set_smem_k(int bytes) {
  return cudaFuncSetAttribute(k_advance<MET, TW>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <int MET, int TW>
void advance_launch_k(int blocks, int threads, size_t smem, cudaStream_t st, const Params& P, const Bufs& B,
                      const DevModel& M, const GradOut& G) {
  k_advance<MET, TW><<<blocks, threads, smem, st>>>(P, B, M, G);
}

template cudaError_t advance_set_smem_k<GNUTS_MET, GNUTS_TW>(int);
template void advance_launch_k<GNUTS_MET, GNUTS_TW>(int, int, size_t, cudaStream_t, const Params&, const Bufs&,
                                                      const DevModel&, const GradOut&);

}  // namespace gnuts
