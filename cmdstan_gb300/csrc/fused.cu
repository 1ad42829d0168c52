// Dispatch of the fused-mode kernel on the model's kind (the per-kind
// instantiations are compiled from fused_kind.cu).
#include <cuda_runtime.h>
#include "internal.h"
#include "nuts_device.cuh"

namespace gnuts {

#define GNUTS_KIND_SWITCH(kind, CALL)            \
  switch (kind) {                                \
    case MK_BERNOULLI: return CALL(MK_BERNOULLI); \
    case MK_NORMAL: return CALL(MK_NORMAL);       \
    case MK_LOGISTIC: return CALL(MK_LOGISTIC);   \
    case MK_HIER: return CALL(MK_HIER);           \
    case MK_FUNNEL: return CALL(MK_FUNNEL);       \
    case MK_VARINT: return CALL(MK_VARINT);       \
    case MK_HORSESHOE: return CALL(MK_HORSESHOE); \
  }                                              \
  return cudaErrorInvalidValue

cudaError_t fused_set_smem(int kind, int bytes) {
#define CALL(K) fused_set_smem_k<K>(bytes)
  GNUTS_KIND_SWITCH(kind, CALL);
#undef CALL
}

cudaError_t fused_launch(int kind, int blocks, int threads, size_t smem, const Params& P, const Bufs& B,
                         const DevModel& M, const ReplayBufs& RB) {
#define CALL(K) fused_launch_k<K>(blocks, threads, smem, P, B, M, RB)
  GNUTS_KIND_SWITCH(kind, CALL);
#undef CALL
}

}  // namespace gnuts
