// The double-float instantiation of the inverse z pass (passes_impl.cuh).
// The form's passes sit in one translation unit each so that they compile in
// parallel (together they take several times longer than apart).
#include "passes_impl.cuh"

namespace samgpu {

SAMGPU_INST_ZINV(dd)

}  // namespace samgpu
