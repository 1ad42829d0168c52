// Host interface of the cuBLASLt batched logistic gradient for wide designs
// (grad_wide.cu).
#pragma once
#include <cuda_runtime.h>
#include <string>
#include "internal.h"

namespace gnuts {

struct GradOut;
struct WidePlan;  // cuBLASLt descriptors, chosen algorithms, workspace, buffers

// logistic or horseshoe model, BF16 X, K and N multiples of 8
bool wide_supported(const DevModel& M);
// Builds the plan for C chains; returns the [C][K+1] FP64 coefficient rows
// that stage_request fills and the [1][C] lp / [1][C][K+1] gradient partials
// that reduce_gradient sums (all owned by the plan).
int wide_create(const DevModel& M, int C, WidePlan** out, double** coef64, double** part_lp, double** part_g,
                std::string& err);
void wide_destroy(WidePlan* p);
// stage -> GEMM1 -> epilogue -> GEMM2 -> partials, all on `st` (capturable)
int wide_launch(const WidePlan* p, const GradOut& G, const DevModel& M, cudaStream_t st);

}  // namespace gnuts
