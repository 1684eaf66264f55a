// Shared declarations of the SAM GB300 device code: grid geometry, the
// device-resident step state, and launch helpers used by every pass.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_engine.cuh"

namespace samgpu {

// Geometry of one run.  Wave space keeps kx in [0, kx_max] (Nx_min modes),
// ky and kz in [-k_max, k_max] stored non-negative first (Ny_min, Nz_min
// modes), as fft_init.f:52-72 orders them.
struct Grid {
  int nx, ny, nz, nze;
  int mx, my, mz;
  int kx, ky, kz;
  int lu, lr;
  double wave_x, wave_y, wave_z;
};

// Scalars the reference keeps in COMMON /dynamic/, /tstep/ and /statistics/
// (sam.h), resident on the device so a step needs no host round trip.
struct DevState {
  double time, dt;
  double u_avg[4], u_var[4], u_max[4];
  double energy, cfl_x, cfl_y, cfl_z;
  int nonfinite;  // set when vel_max meets a NaN/Inf
  int pad;
};

// Per-launch physics constants of one RK stage (sam.f:210-314, rhs.f:108-142).
struct StageConsts {
  int nrk, last, i_strat, rot_sav, i_cfl, write_p;
  double gamma, zeta;
  double vis, pr_inv;
  double buoy_fac_x, buoy_fac_z, lapse, cos_theta, sin_theta;
  double cfl0, adv_cfl_limit;
};

// Signed wave number of stored index j along a direction with k_max = km and
// m = 2 km + 1 stored modes (fft_init.f:57-72).
__device__ __forceinline__ int kwave(int j, int km, int m) { return j <= km ? j : j - m; }

// Position in an FFT line of length n of stored index j (zero band removed).
__device__ __forceinline__ int kpos(int j, int km, int m, int n) { return j <= km ? j : j + (n - m); }

constexpr int kThreads = 256;

// sam_gpu_config.precision of the double-float form (FP32 pairs, about 48
// significand bits; SAM_GPU_PREC_DD in sam_gpu.h)
constexpr int kPrecDD = 48;

// Streaming multiprocessors of the current device (looked up once per
// device): persistent and grid-stride launches are sized in multiples of it.
inline int sm_count() {
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
  if (!cache[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 1;
    cache[dev] = n;
  }
  return cache[dev];
}

// The largest dynamic shared memory a block of the current device may opt
// into (looked up once per device).
inline int smem_optin() {
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
  if (!cache[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || n < 1)
      n = 48 * 1024;
    cache[dev] = n;
  }
  return cache[dev];
}

// Records the message returned by sam_gpu_error_string(); returns code.
int set_error(int code, const char* msg);

}  // namespace samgpu
