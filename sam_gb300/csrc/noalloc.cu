// vel_max without any device allocation.
//
// Some callers cannot call cudaMalloc: a host code that hands the library
// device memory owned by another allocator (a framework's caching pool, a
// Fortran code's preallocated CUDA-aware buffers) and must stay inside that
// allocator's budget, or a time-stepping loop that must not stall, since
// cudaMalloc and cudaFree synchronise the device.  This entry point serves
// them: the caller passes the physical field and the output in device memory,
// and the per-plane partial sums live in a fixed array compiled into the
// library instead of in allocated scratch.
//
// The array is a file-scope __device__ symbol, so every GPU that loads the
// library holds its 512 KB until the process exits.  Its name seen from host
// code is only a host-side stand-in, not a device address: handing it to a
// kernel would fault, or silently touch the wrong memory where the GPU can
// reach host memory.  The device address is therefore looked up with
// cudaGetSymbolAddress once per device, with that device current, on the
// first call made on it; make that first call before any stream capture.
//
// All calls share the one array and each call overwrites every slot it later
// reads, so nothing needs clearing; calls that overlap on the GPU (two streams
// at once) race on it and must be serialised by the caller.
#include <cuda_runtime.h>
#include <math.h>

#include <mutex>

#include "../../include/sam_gpu.h"
#include "common.cuh"

namespace samgpu {

// One row per z plane (at most SAM_GPU_NOALLOC_MAX_PLANES planes), four fields,
// four partials (sum, sum of squares, max |u|, non-finite count).
static __device__ __align__(256) double g_noalloc_partials[SAM_GPU_NOALLOC_MAX_PLANES * 4 * 4];

// vel_max.f:11-21 for one z plane per CTA.
__global__ void k_noalloc_plane_sums(const double* __restrict__ u, long long plane, long long field, int nzp, int lu,
                                     double* __restrict__ part) {
  __shared__ double red[4][kThreads];
  const int k = blockIdx.x;
  for (int f = 0; f < lu; ++f) {
    const double* p = u + f * field + (long long)k * plane;
    double s1 = 0.0, s2 = 0.0, mx = 0.0, bad = 0.0;
    for (long long e = threadIdx.x; e < plane; e += blockDim.x) {
      const double v = p[e];
      s1 += v;
      s2 += v * v;
      mx = fmax(mx, fabs(v));
      bad += isfinite(v) ? 0.0 : 1.0;
    }
    red[0][threadIdx.x] = s1; red[1][threadIdx.x] = s2; red[2][threadIdx.x] = mx; red[3][threadIdx.x] = bad;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
      if (threadIdx.x < h) {
        red[0][threadIdx.x] += red[0][threadIdx.x + h];
        red[1][threadIdx.x] += red[1][threadIdx.x + h];
        red[2][threadIdx.x] = fmax(red[2][threadIdx.x], red[2][threadIdx.x + h]);
        red[3][threadIdx.x] += red[3][threadIdx.x + h];
      }
      __syncthreads();
    }
    if (threadIdx.x < 4) part[((long long)k * 4 + f) * 4 + threadIdx.x] = red[threadIdx.x][0];
    __syncthreads();
  }
}

// vel_max.f:28-34: averages, variances, maxima and energy, summed over the
// planes in a fixed order.
__global__ void k_noalloc_finish(const double* __restrict__ part, int nzp, int lu, double inv_n,
                                 double* __restrict__ out) {
  if (threadIdx.x != 0) return;
  double bad = 0.0;
  for (int f = 0; f < 4; ++f) {
    double s1 = 0.0, s2 = 0.0, mx = 0.0;
    if (f < lu) {
      for (int k = 0; k < nzp; ++k) {
        const double* q = part + ((long long)k * 4 + f) * 4;
        s1 += q[0];
        s2 += q[1];
        mx = fmax(mx, q[2]);
        bad += q[3];
      }
    }
    const double avg = s1 * inv_n;
    out[f] = avg;
    out[4 + f] = f < lu ? s2 * inv_n - avg * avg : 0.0;
    out[8 + f] = mx;
  }
  out[12] = 0.5 * (out[4] + out[5] + out[6]);
  out[13] = bad;
  out[14] = 0.0;
  out[15] = 0.0;
}

static std::mutex g_noalloc_mu;
static double* g_noalloc_ptr[64];  // device address of g_noalloc_partials, per device ordinal

}  // namespace samgpu

using namespace samgpu;

extern "C" int sam_gpu_vel_max_noalloc(const double* u_dev, int nx, int ny, int nzp, int lu, double* stats_dev,
                                       void* stream) {
  if (!u_dev || !stats_dev) return set_error(SAM_GPU_EINVAL, "vel_max_noalloc: null device pointer");
  if (nx < 1 || ny < 1 || nzp < 1 || lu < 1 || lu > 4)
    return set_error(SAM_GPU_EINVAL, "vel_max_noalloc: Nx, Ny, nzp must be >= 1 and Lu in 1..4");
  if (nzp > SAM_GPU_NOALLOC_MAX_PLANES)
    return set_error(SAM_GPU_EINVAL,
                     "vel_max_noalloc: nzp exceeds SAM_GPU_NOALLOC_MAX_PLANES (4096), the compiled-in scratch size");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return set_error(SAM_GPU_ECUDA, "vel_max_noalloc: no current CUDA device");
  double* part = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
      if (e != cudaSuccess || !p) return set_error(SAM_GPU_ECUDA, "vel_max_noalloc: cudaGetSymbolAddress failed");
      g_noalloc_ptr[dev] = (double*)p;
    }
    part = g_noalloc_ptr[dev];
  }
  const long long plane = (long long)nx * ny;
  const long long field = plane * nzp;
  cudaStream_t s = (cudaStream_t)stream;
  k_noalloc_plane_sums<<<nzp, kThreads, 0, s>>>(u_dev, plane, field, nzp, lu, part);
  k_noalloc_finish<<<1, 32, 0, s>>>(part, nzp, lu, 1.0 / ((double)field), stats_dev);
  if (cudaGetLastError() != cudaSuccess) return set_error(SAM_GPU_ECUDA, "vel_max_noalloc: kernel launch failed");
  return SAM_GPU_OK;
}
