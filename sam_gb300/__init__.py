"""GB300-native implementation of SAM's pseudo-spectral RK3 step.

The product is the CUDA library libsam_gpu.so (C ABI in include/sam_gpu.h);
sam_gb300.sam_gpu is its Python host-side mirror and sam_gb300.build compiles
it in-tree for sm_103a.
"""
from .sam_gpu import SamEnsemble, SamGpu, SamGpuError, load_library, reference_config  # noqa: F401
