// The FP64 instantiation of the transform passes (passes_impl.cuh) and the
// precision-independent kernels: vel_max's completion and the x2z layout.
#include "passes_impl.cuh"

namespace samgpu {

template void launch_parseval<float>(const float2*, const Grid&, double*, cudaStream_t);
template void launch_parseval<double>(const double2*, const Grid&, double*, cudaStream_t);

__global__ void k_vel_max_finish(const double* __restrict__ partials, int nblk, Grid g, DevState* st, int i_cfl,
                                 double cfl0, double adv_cfl_limit, const double* __restrict__ pv, int npv,
                                 int* __restrict__ vmax, int vkind) {
  vel_max_finish_body(partials, nblk, g, st, i_cfl, cfl0, adv_cfl_limit, pv, npv, vmax, vkind);
}

// ------------------------------------------------------ x2z layout kernel
// x2z_decomp.f:59-152 with one rank: (Ny_min, Nx_min, Nze, n) blocks to
// (Ny, Nx/2, Nz, n) planes with the truncated ky band zeroed.
__global__ void k_x2z(const double2* __restrict__ in, double2* __restrict__ out, Grid g, int nvar, int nx2) {
  const long long total = (long long)g.ny * g.mx * g.nz * nvar;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(e % g.ny);
    long long r = e / g.ny;
    const int i = (int)(r % g.mx);
    r /= g.mx;
    const int k = (int)(r % g.nz);
    const int n = (int)(r / g.nz);
    double2 v = make_double2(0.0, 0.0);
    int j = -1;
    if (y <= g.ky) j = y;
    else if (y >= g.ny - g.ky) j = y - (g.ny - g.my);
    if (j >= 0) v = in[(((long long)n * g.nze + k) * g.mx + i) * g.my + j];
    out[(((long long)n * g.nz + k) * nx2 + i) * g.ny + y] = v;
  }
}

void launch_vel_max_finish(const double* partials, int nblk, const Grid& g, DevState* st, int i_cfl, double cfl0,
                           double adv_cfl_limit, cudaStream_t s, const double* pv, int npv, int* vmax, int vkind) {
  k_vel_max_finish<<<1, kThreads, 0, s>>>(partials, nblk, g, st, i_cfl, cfl0, adv_cfl_limit, pv, npv, vmax, vkind);
}
void launch_x2z(const double2* in, double2* out, const Grid& g, int nvar, int nx2, cudaStream_t s) {
  long long total = (long long)g.ny * g.mx * g.nz * nvar;
  int grid = (int)((total + kThreads - 1) / kThreads);
  if (grid > sm_count() * 16) grid = sm_count() * 16;
  if (grid < 1) grid = 1;
  k_x2z<<<grid, kThreads, 0, s>>>(in, out, g, nvar, nx2);
}


SAMGPU_INST(double)

}  // namespace samgpu
