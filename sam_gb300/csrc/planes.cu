// Planes output path: the wave-space fields that sam.f:145-166 loads into r
// at output steps, and the plane cuts write_planes.f writes.
#include "planes.cuh"

namespace samgpu {

static int blocks_for(long long n) {
  long long b = (n + kThreads - 1) / kThreads;
  if (b > sm_count() * 32) b = sm_count() * 32;
  return (int)(b < 1 ? 1 : b);
}

// sam.f:150-160: r(Lu+1) = p, r(Lu+1+m) = i wave_z k_z u(m); write_planes.f
// differentiates in y (y_deriv.f) and x (x_deriv.f), done here as i k times
// the band-limited spectrum, which is what those routines compute.
template <typename T>
__global__ void k_planes_fields(Grid g, PlaneFields pf, const cx_t<T>* __restrict__ u, const cx_t<T>* __restrict__ p,
                                cx_t<T>* __restrict__ w) {
  using C = cx_t<T>;
  const long long nm = (long long)g.mx * g.my * g.mz;
  const long long total = nm * pf.nf;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int f = (int)(e / nm);
    const long long r = e - (long long)f * nm;
    const int kz = (int)(r % g.mz);
    const int ky = (int)((r / g.mz) % g.my);
    const int kx = (int)(r / ((long long)g.mz * g.my));
    const int src = pf.src[f], op = pf.op[f];
    const C v = src < 0 ? p[r] : u[(long long)src * nm + r];
    double b;
    if (op == 0) {
      w[e] = v;
      continue;
    } else if (op == 1) {
      b = g.wave_z * (double)kwave(kz, g.kz, g.mz);
    } else if (op == 2) {
      b = g.wave_y * (double)kwave(ky, g.ky, g.my);
    } else {
      b = g.wave_x * (double)kx;
    }
    const T bt = (T)b;
    w[e] = mk<C>(-bt * v.y, bt * v.x);
  }
}

template <typename T>
__global__ void k_planes_gather(Grid g, PlaneSel sel, const T* __restrict__ ph, double* __restrict__ xy,
                                double* __restrict__ xz, double* __restrict__ yz) {
  const long long pl = (long long)g.nx * g.ny;
  const long long vol = pl * g.nz;
  const long long nxy = (long long)sel.n_xy * sel.n_out * pl;
  const long long nxz = (long long)sel.n_xz * sel.n_out * g.nx * g.nz;
  const long long nyz = (long long)sel.n_yz * sel.n_out * g.ny * g.nz;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nxy + nxz + nyz;
       e += (long long)gridDim.x * blockDim.x) {
    if (e < nxy) {  // xy(x, y, slot, m) = uu(x, y, k_xy(m), slot)
      const long long q = e / pl, r = e - q * pl;
      const int s = (int)(q % sel.n_out), m = (int)(q / sel.n_out);
      xy[e] = (double)ph[(long long)sel.fxy[s] * vol + (long long)sel.k_xy[m] * pl + r];
    } else if (e < nxy + nxz) {  // xz(x, z, slot, m) = uu(x, j_xz(m), z, .)
      const long long e2 = e - nxy;
      const int x = (int)(e2 % g.nx);
      const long long q = e2 / g.nx;
      const int z = (int)(q % g.nz);
      const long long q2 = q / g.nz;
      const int s = (int)(q2 % sel.n_out), m = (int)(q2 / sel.n_out);
      xz[e2] = (double)ph[(long long)sel.fxz[s] * vol + (long long)z * pl + (long long)sel.j_xz[m] * g.nx + x];
    } else {  // yz(y, z, slot, m) = uu(i_yz(m), y, z, .)
      const long long e3 = e - nxy - nxz;
      const int y = (int)(e3 % g.ny);
      const long long q = e3 / g.ny;
      const int z = (int)(q % g.nz);
      const long long q2 = q / g.nz;
      const int s = (int)(q2 % sel.n_out), m = (int)(q2 / sel.n_out);
      yz[e3] = (double)ph[(long long)sel.fyz[s] * vol + (long long)z * pl + (long long)y * g.nx + sel.i_yz[m]];
    }
  }
}

template <typename T>
void planes_fields(const Grid& g, const PlaneFields& pf, const cx_t<T>* u, const cx_t<T>* p, cx_t<T>* w,
                   cudaStream_t s) {
  const long long n = (long long)g.mx * g.my * g.mz * pf.nf;
  k_planes_fields<T><<<blocks_for(n), kThreads, 0, s>>>(g, pf, u, p, w);
}

template <typename T>
void planes_gather(const Grid& g, const PlaneSel& sel, const T* ph, double* xy, double* xz, double* yz,
                   cudaStream_t s) {
  const long long n = ((long long)sel.n_xy * g.nx * g.ny + (long long)sel.n_xz * g.nx * g.nz +
                       (long long)sel.n_yz * g.ny * g.nz) * sel.n_out;
  if (n == 0) return;
  k_planes_gather<T><<<blocks_for(n), kThreads, 0, s>>>(g, sel, ph, xy, xz, yz);
}

template void planes_fields<float>(const Grid&, const PlaneFields&, const float2*, const float2*, float2*,
                                   cudaStream_t);
template void planes_fields<double>(const Grid&, const PlaneFields&, const double2*, const double2*, double2*,
                                    cudaStream_t);
template void planes_gather<float>(const Grid&, const PlaneSel&, const float*, double*, double*, double*,
                                   cudaStream_t);
template void planes_gather<double>(const Grid&, const PlaneSel&, const double*, double*, double*, double*,
                                    cudaStream_t);
}  // namespace samgpu
