// The double-float instantiation of the forward y pass (passes_impl.cuh).
#include "passes_impl.cuh"

namespace samgpu {

SAMGPU_INST_YFWD(dd)

}  // namespace samgpu
