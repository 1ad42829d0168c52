// Round-mode state-machine step k_advance: defined in advance_kind.cu, which
// is compiled once per (metric, team width) so the instantiations build in
// parallel and each carries only its own metric's code.
#pragma once
#include <cuda_runtime.h>
#include "nuts_device.cuh"
#include "batched.cuh"

namespace gnuts {

// chains of at least TEAM_MIN_D parameters advance as CTA teams of TEAM_TW
// threads (252-254 registers per thread: two teams per SM)
constexpr int TEAM_MIN_D = 512;
constexpr int TEAM_TW = 128;

template <int MET, int TW>
cudaError_t advance_set_smem_k(int bytes);
template <int MET, int TW>
void advance_launch_k(int blocks, int threads, size_t smem, cudaStream_t st, const Params& P, const Bufs& B,
                      const DevModel& M, const GradOut& G);

}  // namespace gnuts
