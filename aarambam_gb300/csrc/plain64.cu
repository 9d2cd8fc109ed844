// Plain FP64 form of the IC path: cuFFT Z2D / D2Z transforms and separate
// pointwise kernels, loop structure 1:1 with the reference
// (Aarambam/LPT/Basis/main.c:564-1516).
#include <cuda_runtime.h>

#include "aar_internal.cuh"

namespace aar {

int plain_run(Plan* p, const float*, int64_t, float*, float*, cudaStream_t) {
  return set_err(p, "plain FP64 form not built yet"), AAR_ERR_ARG;
}
void plain_free(Plan*) {}

}  // namespace aar
