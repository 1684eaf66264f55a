// The double-float instantiation of the x pass and of vel_max's wave-space
// sums (passes_impl.cuh).
#include "passes_impl.cuh"

namespace samgpu {

SAMGPU_INST_X(dd)
template void launch_parseval<dd>(const ddc*, const Grid&, double*, cudaStream_t);

}  // namespace samgpu
