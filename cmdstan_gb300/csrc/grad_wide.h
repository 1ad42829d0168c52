// Host interface of the tcgen05 batched logistic gradient for wide designs
// (grad_wide.cu).
#pragma once
#include <cuda_runtime.h>
#include <string>
#include "internal.h"

namespace gnuts {

struct GradOut;
struct WidePlan;  // tensor maps, grids and buffers of the two tensor-core kernels

// logistic or horseshoe model, BF16 X and packed y, K a multiple of 8
bool wide_supported(const DevModel& M);
// Builds the plan for C chains; returns the [C][K+1] FP64 coefficient rows
// that stage_request fills and the [1][C] lp / [1][C][K+1] gradient partials
// that reduce_gradient sums (all owned by the plan).
// The kernels return at once when *done_count reaches C (round mode).
int wide_create(const DevModel& M, int C, const int* done_count, WidePlan** out, double** coef64,
                double** part_lp, double** part_g, std::string& err);
void wide_destroy(WidePlan* p);
// stage -> k_wide_eta -> k_wide_xtr -> partials, all on `st` (capturable)
int wide_launch(const WidePlan* p, const GradOut& G, const DevModel& M, cudaStream_t st);
// nonzero when a kernel's bounded wait expired (synchronises)
int wide_error(const WidePlan* p);

}  // namespace gnuts
