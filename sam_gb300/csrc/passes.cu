// The FP64 instantiation of the transform passes (passes_impl.cuh) and the
// precision-independent kernels: vel_max's completion and the x2z layout.
#include "passes_impl.cuh"

namespace samgpu {

template void launch_parseval<float>(const float2*, const Grid&, double*, cudaStream_t);
template void launch_parseval<double>(const double2*, const Grid&, double*, cudaStream_t);

__global__ void k_vel_max_finish(const double* __restrict__ partials, int nblk, Grid g, DevState* st, int i_cfl,
                                 double cfl0, double adv_cfl_limit, const double* __restrict__ pv, int npv,
                                 int* __restrict__ vmax, int vkind) {
  __shared__ double red[kThreads];
  __shared__ double fin[4][4];
  if (!pv) {
    // a thread reads whole per-CTA records (lu x 4 doubles, contiguous) of
    // the CTAs b = t, t + 256, ... into 16 accumulators, then one fixed-order
    // tree per quantity: deterministic for a given number of CTAs
    __shared__ double redq[16][kThreads / 2];
    double v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = 0.0;
    const int nq = 4 * g.lu;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
      const double2* rec = reinterpret_cast<const double2*>(partials + (long long)b * nq);
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (2 * i < nq) {
          const double2 x = rec[i];
          v[2 * i] = ((2 * i) % 4 == 2) ? fmax(v[2 * i], x.x) : v[2 * i] + x.x;
          v[2 * i + 1] = ((2 * i + 1) % 4 == 2) ? fmax(v[2 * i + 1], x.y) : v[2 * i + 1] + x.y;
        }
    }
    // first tree level straight from the registers (threads t and t + 128)
    const int h = blockDim.x / 2;
    if (threadIdx.x >= h)
#pragma unroll
      for (int i = 0; i < 16; ++i) redq[i][threadIdx.x - h] = v[i];
    __syncthreads();
    if (threadIdx.x < h)
#pragma unroll
      for (int i = 0; i < 16; ++i)
        redq[i][threadIdx.x] = (i % 4 == 2) ? fmax(v[i], redq[i][threadIdx.x]) : v[i] + redq[i][threadIdx.x];
    __syncthreads();
    for (int st = h / 2; st > 0; st >>= 1) {
      if (threadIdx.x < st)
#pragma unroll
        for (int i = 0; i < 16; ++i)
          redq[i][threadIdx.x] = (i % 4 == 2) ? fmax(redq[i][threadIdx.x], redq[i][threadIdx.x + st])
                                              : redq[i][threadIdx.x] + redq[i][threadIdx.x + st];
      __syncthreads();
    }
    if (threadIdx.x < nq) fin[threadIdx.x / 4][threadIdx.x % 4] = redq[threadIdx.x][0];
    __syncthreads();
  }
  if (pv) {
    // sums from wave space: sum u = N u(0,0,0), sum u^2 = N sum w |u|^2
    for (int f = 0; f < g.lu; ++f) {
      double v = 0.0;
      for (int b = threadIdx.x; b < npv; b += blockDim.x) v += pv[(long long)b * g.lu + f];
      red[threadIdx.x] = v;
      __syncthreads();
      for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        const double n = (double)g.nx * (double)g.ny * (double)g.nz;
        fin[f][0] = pv[(long long)npv * g.lu + f] * n;
        fin[f][1] = red[0] * n;
        fin[f][2] = vkind ? dd_key_value(reinterpret_cast<const unsigned long long*>(vmax)[f])
                          : (double)__int_as_float(vmax[f]);
        fin[f][3] = (double)vmax[8];
      }
      __syncthreads();
    }
    __syncthreads();
    if (threadIdx.x < kVmaxInts) vmax[threadIdx.x] = 0;  // ready for the next step's maxima
  }
  if (threadIdx.x == 0) {
    const double inv = 1.0 / ((double)g.nx * (double)g.ny * (double)g.nz);
    int bad = 0;
    for (int f = 0; f < g.lu; ++f) {
      st->u_avg[f] = fin[f][0] * inv;
      st->u_var[f] = fin[f][1] * inv - st->u_avg[f] * st->u_avg[f];
      st->u_max[f] = fin[f][2];
      bad |= fin[f][3] != 0.0;
    }
    st->energy = 0.5 * (st->u_var[0] + st->u_var[1] + st->u_var[2]);
    const double cx = st->u_max[0] * g.kx * g.wave_x;
    const double cy = st->u_max[1] * g.ky * g.wave_y;
    const double cz = st->u_max[2] * g.kz * g.wave_z;
    if (i_cfl == 1) {
      const double cb = fmax(cx, fmax(cy, cz));
      if (cb > 0.0 && !bad) st->dt = cfl0 * adv_cfl_limit / cb;
    }
    st->cfl_x = cx * st->dt;
    st->cfl_y = cy * st->dt;
    st->cfl_z = cz * st->dt;
    if (bad) st->nonfinite = 1;
  }
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
