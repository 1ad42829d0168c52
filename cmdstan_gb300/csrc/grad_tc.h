// Host interface of the tcgen05 batched logistic gradient (grad_tc.cu).
#pragma once
#include <cuda_runtime.h>
#include <string>
#include "internal.h"

namespace gnuts {

struct TcPlan;  // tensor maps, buffers, launch shape

// Builds the plan for C chains of a logistic model with K + 1 <= 128.
// coef_bf (returned) is the [2][Cpad][128] BF16 hi/lo coefficient buffer that
// stage_request fills; part_lp is [S][C] FP64, part_g [S][C][TC_GSTRIDE] FP32
// (position k < K: beta_k, position K: intercept); lin is [C] FP64, the
// linear likelihood part that stage_request writes and reduce_gradient adds.
int tc_create(const DevModel& M, int C, const int* done_count, TcPlan** plan, uint16_t** coef_bf, int* S,
              double** part_lp, float** part_g, double** lin, std::string& err);
void tc_destroy(TcPlan* plan);
bool tc_supported(const DevModel& M);
void tc_launch(const TcPlan* plan, cudaStream_t stream);
// non-zero if a bounded wait inside the kernel ran out since the last reset
int tc_error(const TcPlan* plan);

}  // namespace gnuts
