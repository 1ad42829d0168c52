// Tensor-core (tcgen05) contraction for the batched logistic gradient.
// Placeholder translation unit; the kernel lands here.
#include "internal.h"
