// The double-float instantiation of the inverse y pass (passes_impl.cuh).
#include "passes_impl.cuh"

namespace samgpu {

SAMGPU_INST_YINV(dd)

}  // namespace samgpu
