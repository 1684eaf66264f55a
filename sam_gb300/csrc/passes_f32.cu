// The FP32 instantiation of the transform passes (passes_impl.cuh).
#include "passes_impl.cuh"

namespace samgpu {

SAMGPU_INST(float)

}  // namespace samgpu
