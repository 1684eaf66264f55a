// Subgrid-model routines of the reference (filter.f, sm.f, dm.f) and the
// mean-profile routine get_mean.f, in FP64 on haloed (Nx+2, Ny+2, Nz+2) grids.
//
// filter.f, sm.f and dm.f include a header the reference does not ship
// (speciso.h).  Its symbols are defined from their use:
//   Lx = Nx+2, Ly = Ny+2, Lz = Nz+2: planes 1 and N+2 are periodic halos
//     (periodicity.f:7-32);
//   ifact = (1,1,1,2,2,2) over the symmetric tensor (S11,S22,S33,S12,S23,S13);
//   ip = (1,2,3,1,2,1), jp = (1,2,3,2,3,3): index pairs of that tensor;
//   alpha_sq = 4: (test/grid filter width)^2 for the 1-4-1 test filter;
//   delta_sq = (dx dy dz)^(2/3) (init.f:28).
// The plane-by-plane sweeps of sm.f and dm.f become stencils over the whole
// volume: with periodic halos in the input every plane slot they read is the
// periodic neighbour of the plane being processed, so each point can be
// computed independently.
#include <cuda_runtime.h>
#include <math.h>

#include "common.cuh"
#include "les.cuh"

namespace samgpu {

struct Halo {
  int nx, ny, nz;
  __device__ __forceinline__ long long at(int i, int j, int k) const {
    return (long long)i + (long long)(nx + 2) * ((long long)j + (long long)(ny + 2) * k);
  }
  __device__ __forceinline__ long long vol() const { return (long long)(nx + 2) * (ny + 2) * (nz + 2); }
  // interior (periodic) index 0..n-1 of a wrapped coordinate; the stencils
  // reach one point past either side, so a conditional add or subtract
  // replaces the integer remainder (valid for -n <= i < 2n)
  __device__ __forceinline__ static int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
  __device__ __forceinline__ int wx(int i) const { return wrap(i, nx); }
  __device__ __forceinline__ int wy(int j) const { return wrap(j, ny); }
  __device__ __forceinline__ int wz(int k) const { return wrap(k, nz); }
  __device__ __forceinline__ long long in(int i, int j, int k) const {
    return (long long)wx(i) + (long long)nx * ((long long)wy(j) + (long long)ny * wz(k));
  }
  __device__ __forceinline__ long long ninterior() const { return (long long)nx * ny * nz; }
};

__constant__ int c_ifact[6] = {1, 1, 1, 2, 2, 2};
__constant__ int c_ip[6] = {0, 1, 2, 0, 1, 0};
__constant__ int c_jp[6] = {0, 1, 2, 1, 2, 2};

// ---- filter.f:7-42 on one 2-D plane set: 1-4-1 across the three planes of
// f_bar(Lx,Ly,n_var,3) (halos included), 1-4-1 along y using those halo rows,
// then along x with periodic wrap, normalised by 1/6^3; halos periodic.
__global__ void k_filter(const double* __restrict__ f_bar, double* __restrict__ f_hat, int nx, int ny, int n_var) {
  const int lx = nx + 2, ly = ny + 2;
  const long long pl = (long long)lx * ly;
  const long long tot = (long long)lx * ly * n_var;
  const double w_inv = 1.0 / (6.0 * 6.0 * 6.0);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % lx), j = (int)((e / lx) % ly), n = (int)(e / pl);
    // the value at halo points is the periodic image of the interior result
    const int ii = i == 0 ? nx : (i == nx + 1 ? 1 : i);
    const int jj = j == 0 ? ny : (j == ny + 1 ? 1 : j);
    auto h = [&](int a, int b) {
      const long long o = (long long)a + (long long)lx * b + pl * n;
      return f_bar[o] + 4 * f_bar[o + pl * n_var] + f_bar[o + 2 * pl * n_var];
    };
    auto g = [&](int a) { return h(a, jj - 1) + 4 * h(a, jj) + h(a, jj + 1); };
    const int am = ii - 1 == 0 ? nx : ii - 1;  // periodic wrap of the y-filtered rows
    const int ap = ii + 1 == nx + 1 ? 1 : ii + 1;
    f_hat[e] = w_inv * (g(am) + 4 * g(ii) + g(ap));
  }
}

// ---- staggered-to-centre velocity u_bar on the interior (sm.f:47-49)
__global__ void k_ubar(const double* __restrict__ u, double* __restrict__ ub, Halo H) {
  const long long n = H.ninterior(), vol = H.vol();
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % H.nx) + 1, j = (int)((e / H.nx) % H.ny) + 1, k = (int)(e / ((long long)H.nx * H.ny)) + 1;
    ub[e] = 0.5 * (u[H.at(i, j, k)] + u[H.at(i - 1, j, k)]);
    ub[n + e] = 0.5 * (u[vol + H.at(i, j, k)] + u[vol + H.at(i, j - 1, k)]);
    ub[2 * n + e] = 0.5 * (u[2 * vol + H.at(i, j, k)] + u[2 * vol + H.at(i, j, k - 1)]);
  }
}

// strain (sm.f:57-75) at interior point (x, y, z) from periodic u_bar
__device__ __forceinline__ void strain(const double* __restrict__ ub, const Halo& H, int x, int y, int z, double dxi,
                                       double dyi, double dzi, double* s) {
  const long long n = H.ninterior();
  auto U = [&](int c, int a, int b, int d) { return ub[c * n + H.in(a, b, d)]; };
  s[0] = 0.5 * (U(0, x + 1, y, z) - U(0, x - 1, y, z)) * dxi;
  s[1] = 0.5 * (U(1, x, y + 1, z) - U(1, x, y - 1, z)) * dyi;
  s[2] = 0.5 * (U(2, x, y, z + 1) - U(2, x, y, z - 1)) * dzi;
  s[3] = .25 * ((U(0, x, y + 1, z) - U(0, x, y - 1, z)) * dyi + (U(1, x + 1, y, z) - U(1, x - 1, y, z)) * dxi);
  s[4] = .25 * ((U(1, x, y, z + 1) - U(1, x, y, z - 1)) * dzi + (U(2, x, y + 1, z) - U(2, x, y - 1, z)) * dyi);
  s[5] = .25 * ((U(2, x + 1, y, z) - U(2, x - 1, y, z)) * dxi + (U(0, x, y, z + 1) - U(0, x, y, z - 1)) * dzi);
}

__device__ __forceinline__ double smag(const double* s) {
  double sum = 0.0;
  for (int q = 0; q < 6; ++q) sum += c_ifact[q] * s[q] * s[q];
  return sqrt(2.0 * sum);
}

// sm.f:77-86: vt = c_smag delta^2 |S| on the interior of the haloed output
__global__ void k_sm(const double* __restrict__ ub, double* __restrict__ vt, Halo H, double c_delta_sq, double dxi,
                     double dyi, double dzi) {
  const long long n = H.ninterior();
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(e % H.nx), y = (int)((e / H.nx) % H.ny), z = (int)(e / ((long long)H.nx * H.ny));
    double s[6];
    strain(ub, H, x, y, z, dxi, dyi, dzi, s);
    vt[H.at(x + 1, y + 1, z + 1)] = c_delta_sq * smag(s);
  }
}

// periodicity.f:7-32 on a haloed volume (every halo point from its image)
__global__ void k_periodic3(double* __restrict__ f, Halo H) {
  const long long tot = H.vol();
  const int lx = H.nx + 2, ly = H.ny + 2;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % lx), j = (int)((e / lx) % ly), k = (int)(e / ((long long)lx * ly));
    const bool halo = i == 0 || i == H.nx + 1 || j == 0 || j == H.ny + 1 || k == 0 || k == H.nz + 1;
    if (!halo) continue;
    const int ii = i == 0 ? H.nx : (i == H.nx + 1 ? 1 : i);
    const int jj = j == 0 ? H.ny : (j == H.ny + 1 ? 1 : j);
    const int kk = k == 0 ? H.nz : (k == H.nz + 1 ? 1 : k);
    f[e] = f[H.at(ii, jj, kk)];
  }
}

// dm.f:99-116: |S|, |S| S_ij and u_bar_i u_bar_j on the interior
//   q[0..5] = S, q[6..11] = |S| S, q[12..17] = ub_i ub_j, q[18] = |S|
__global__ void k_dm_fields(const double* __restrict__ ub, double* __restrict__ q, Halo H, double dxi, double dyi,
                            double dzi) {
  const long long n = H.ninterior();
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(e % H.nx), y = (int)((e / H.nx) % H.ny), z = (int)(e / ((long long)H.nx * H.ny));
    double s[6];
    strain(ub, H, x, y, z, dxi, dyi, dzi, s);
    const double sm = smag(s);
    for (int c = 0; c < 6; ++c) {
      q[c * n + e] = s[c];
      q[(6 + c) * n + e] = sm * s[c];
      q[(12 + c) * n + e] = ub[c_ip[c] * n + e] * ub[c_jp[c] * n + e];
    }
    q[18 * n + e] = sm;
  }
}

// separable 1-4-1 test filter of one periodic interior field at (x, y, z),
// summed in filter.f's order: across planes, then along y, then along x
__device__ __forceinline__ double tfilter(const double* __restrict__ f, const Halo& H, int x, int y, int z) {
  auto h = [&](int a, int b) {
    return f[H.in(x + a, y + b, z - 1)] + 4 * f[H.in(x + a, y + b, z)] + f[H.in(x + a, y + b, z + 1)];
  };
  auto g = [&](int a) { return h(a, -1) + 4 * h(a, 0) + h(a, 1); };
  return (1.0 / 216.0) * (g(-1) + 4 * g(0) + g(1));
}

// dm.f:122-150: L_ij, M_ij at each interior point, per-CTA sums of
// ifact L M and ifact M M (fixed-order tree, deterministic)
__global__ void k_dm_lm(const double* __restrict__ ub, const double* __restrict__ q, Halo H, double alpha_sq,
                        double* __restrict__ part) {
  __shared__ double red[2][kThreads];
  const long long n = H.ninterior();
  double num = 0.0, den = 0.0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(e % H.nx), y = (int)((e / H.nx) % H.ny), z = (int)(e / ((long long)H.nx * H.ny));
    double uh[3], sh[6];
    for (int c = 0; c < 3; ++c) uh[c] = tfilter(ub + c * n, H, x, y, z);
    for (int c = 0; c < 6; ++c) sh[c] = tfilter(q + c * n, H, x, y, z);
    const double smh = smag(sh);
    for (int c = 0; c < 6; ++c) {
      const double M = -tfilter(q + (6 + c) * n, H, x, y, z) + alpha_sq * smh * sh[c];
      const double L = tfilter(q + (12 + c) * n, H, x, y, z) - uh[c_ip[c]] * uh[c_jp[c]];
      num += c_ifact[c] * L * M;
      den += c_ifact[c] * M * M;
    }
  }
  red[0][threadIdx.x] = num;
  red[1][threadIdx.x] = den;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      red[0][threadIdx.x] += red[0][threadIdx.x + h];
      red[1][threadIdx.x] += red[1][threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = red[0][0];
    part[2 * blockIdx.x + 1] = red[1][0];
  }
}

// dm.f:176 and 183-189: c_delta_sq = -num / (2 den); vt = c_delta_sq |S|
__global__ void k_dm_finish(const double* __restrict__ part, int nblk, double* __restrict__ cds) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double num = 0.0, den = 0.0;
    for (int b = 0; b < nblk; ++b) {
      num += part[2 * b];
      den += part[2 * b + 1];
    }
    cds[0] = -0.5 * num / den;
  }
}

__global__ void k_dm_vt(const double* __restrict__ q, const double* __restrict__ cds, double* __restrict__ vt, Halo H) {
  const long long n = H.ninterior();
  const double c = cds[0];
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(e % H.nx), y = (int)((e / H.nx) % H.ny), z = (int)(e / ((long long)H.nx * H.ny));
    vt[H.at(x + 1, y + 1, z + 1)] = c * q[18 * n + e];
  }
}

// ---- get_mean.f:8-56 (i_symm = 0) on the kx = ky = 0 column.  One CTA;
// line 0 of the shared tile holds the synthesis, line 1 the linear profile.
__global__ void k_get_mean(double2* __restrict__ col, int mz, int kz, int nz, int i_remove,
                           const FftPlan* __restrict__ gpl, const double2* __restrict__ gtw,
                           double* __restrict__ u_mean, double* __restrict__ jump_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ FftPlan pl;
  __shared__ double s_jump;
  load_plan(&pl, gpl);
  __syncthreads();
  const int ld = line_stride(nz);
  double2* s_tw = reinterpret_cast<double2*>(smem_raw);
  double2* ln = s_tw + pl.tw_total;
  for (int e = threadIdx.x; e < pl.tw_total; e += blockDim.x) s_tw[e] = gtw[e];
  const double nz_inv = 1.0 / nz;
  for (int pass = 0; pass < 2; ++pass) {
    // rfftb of the packed profile: u_mean(1) = Re u(1), (2k-2, 2k-1) = u(k),
    // k = 2..kz_max+1; as a complex synthesis with the Hermitian extension
    for (int p = threadIdx.x; p < nz; p += blockDim.x) {
      double2 v = make_double2(0.0, 0.0);
      if (p == 0) v = make_double2(col[0].x, 0.0);
      else if (p <= kz) v = col[p];
      else if (p >= nz - kz) v = make_double2(col[nz - p].x, -col[nz - p].y);
      ln[sidx(p)] = v;
    }
    __syncthreads();
    fft_lines<+1>(ln, ld, 1, s_tw, pl);
    __syncthreads();
    if (threadIdx.x == 0) {
      const double m0 = ln[sidx(0)].x, m1 = ln[sidx(1 % nz)].x, m2 = ln[sidx(2 % nz)].x;
      const double l0 = ln[sidx(nz - 1)].x, l1 = ln[sidx((nz - 2 + nz) % nz)].x, l2 = ln[sidx((nz - 3 + nz) % nz)].x;
      const double u_n = 3.0 * m0 - 3.0 * m1 + m2;
      const double u_1 = 3.0 * l0 - 3.0 * l1 + l2;
      const double jmp = 0.5 * ((l0 - u_n) + (u_1 - m0));
      if (pass == 0) s_jump = jmp;
      else s_jump = s_jump - jmp;
    }
    for (int p = threadIdx.x; p < nz; p += blockDim.x) u_mean[p] = ln[sidx(p)].x;
    __syncthreads();
    if (pass == 1 || i_remove != 1) break;
    // the linear profile jump (k/Nz - 1/2), rfftf, and its first kz_max+1
    // packed entries scaled by 1/Nz (get_mean.f:24-32)
    const double jump = s_jump;
    __syncthreads();
    for (int p = threadIdx.x; p < nz; p += blockDim.x) ln[sidx(p)] = make_double2(jump * ((double)p * nz_inv - 0.5), 0.0);
    __syncthreads();
    fft_lines<-1>(ln, ld, 1, s_tw, pl);
    __syncthreads();
    if (threadIdx.x == 0) {
      // packed r(0) = X0, r(2k-1) = Re Xk, r(2k) = Im Xk (0-based)
      auto packed = [&](int idx) {
        if (idx == 0) return ln[sidx(0)].x;
        const int k = (idx + 1) / 2;
        return (idx % 2 == 1) ? ln[sidx(k)].x : ln[sidx(k)].y;
      };
      auto scaled = [&](int idx) { return idx <= kz ? packed(idx) * nz_inv : packed(idx); };
      col[0].x -= scaled(0);
      for (int k = 1; k <= kz; ++k) {
        const double wr = scaled(2 * k - 1), wi = scaled(2 * k);
        const int k2 = mz - k;
        col[k].x -= wr;
        col[k].y -= wi;
        col[k2].x -= wr;
        col[k2].y += wi;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) jump_out[0] = s_jump;
}

static int grid_of(long long n) {
  long long g = (n + kThreads - 1) / kThreads;
  if (g > sm_count() * 16) g = sm_count() * 16;
  return (int)(g < 1 ? 1 : g);
}

void les_filter(const double* f_bar, double* f_hat, int nx, int ny, int n_var, cudaStream_t s) {
  k_filter<<<grid_of((long long)(nx + 2) * (ny + 2) * n_var), kThreads, 0, s>>>(f_bar, f_hat, nx, ny, n_var);
}

static Halo halo(int nx, int ny, int nz) {
  Halo H;
  H.nx = nx; H.ny = ny; H.nz = nz;
  return H;
}

void les_sm(const double* u, double* ub, double* vt, int nx, int ny, int nz, double c_delta_sq, double dxi, double dyi,
            double dzi, cudaStream_t s) {
  const Halo H = halo(nx, ny, nz);
  const long long n = (long long)nx * ny * nz;
  k_ubar<<<grid_of(n), kThreads, 0, s>>>(u, ub, H);
  k_sm<<<grid_of(n), kThreads, 0, s>>>(ub, vt, H, c_delta_sq, dxi, dyi, dzi);
  k_periodic3<<<grid_of((long long)(nx + 2) * (ny + 2) * (nz + 2)), kThreads, 0, s>>>(vt, H);
}

int les_dm_blocks(int nx, int ny, int nz) { return grid_of((long long)nx * ny * nz); }

void les_dm(const double* u, double* ub, double* q, double* part, double* cds, double* vt, int nx, int ny, int nz,
            double alpha_sq, double dxi, double dyi, double dzi, cudaStream_t s) {
  const Halo H = halo(nx, ny, nz);
  const long long n = (long long)nx * ny * nz;
  const int nb = grid_of(n);
  k_ubar<<<nb, kThreads, 0, s>>>(u, ub, H);
  k_dm_fields<<<nb, kThreads, 0, s>>>(ub, q, H, dxi, dyi, dzi);
  k_dm_lm<<<nb, kThreads, 0, s>>>(ub, q, H, alpha_sq, part);
  k_dm_finish<<<1, 32, 0, s>>>(part, nb, cds);
  k_dm_vt<<<nb, kThreads, 0, s>>>(q, cds, vt, H);
  k_periodic3<<<grid_of((long long)(nx + 2) * (ny + 2) * (nz + 2)), kThreads, 0, s>>>(vt, H);
}

// ---- coupled dynamic closure: the physical velocity P(n, z, y, x) of the
// x pass (working precision) into dm.f's haloed FP64 layout u(Lx,Ly,Lz,3),
// halo planes filled with the periodic images (periodicity.f:7-32)
template <typename T>
__global__ void k_pack_halo(const T* __restrict__ phys, double* __restrict__ uh, Halo H) {
  const long long vol = H.vol(), tot = 3 * vol;
  const int lx = H.nx + 2, ly = H.ny + 2;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int n = (int)(e / vol);
    const long long r = e - n * vol;
    const int i = (int)(r % lx), j = (int)((r / lx) % ly), k = (int)(r / ((long long)lx * ly));
    uh[e] = (double)phys[(long long)n * H.ninterior() + H.in(i - 1, j - 1, k - 1)];
  }
}

// C delta^2 in use: dm.f's value, or 0 where it is negative (backscatter
// would make the eddy viscosity negative) or undefined (no strain: 0/0)
__global__ void k_les_clip(const double* __restrict__ raw, double* __restrict__ cds) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const double v = raw[0];
    cds[0] = v > 0.0 ? v : 0.0;
  }
}

size_t les_dynamic_work(int nx, int ny, int nz) {
  const size_t n = (size_t)nx * ny * nz, vol = (size_t)(nx + 2) * (ny + 2) * (nz + 2);
  return 4 * vol + 22 * n + 2 * (size_t)les_dm_blocks(nx, ny, nz) + 8;
}

template <typename T>
void les_dynamic(const T* phys, double* work, double* cds, int nx, int ny, int nz, double dxi, double dyi,
                 double dzi, cudaStream_t s) {
  const Halo H = halo(nx, ny, nz);
  const size_t n = (size_t)nx * ny * nz, vol = (size_t)(nx + 2) * (ny + 2) * (nz + 2);
  double* uh = work;
  double* vt = uh + 3 * vol;
  double* ub = vt + vol;
  double* q = ub + 3 * n;
  double* part = q + 19 * n;
  double* raw = part + 2 * les_dm_blocks(nx, ny, nz);
  k_pack_halo<T><<<grid_of(3 * (long long)vol), kThreads, 0, s>>>(phys, uh, H);
  les_dm(uh, ub, q, part, raw, vt, nx, ny, nz, 4.0, dxi, dyi, dzi, s);
  k_les_clip<<<1, 32, 0, s>>>(raw, cds);
}
template void les_dynamic<double>(const double*, double*, double*, int, int, int, double, double, double,
                                  cudaStream_t);
template void les_dynamic<float>(const float*, double*, double*, int, int, int, double, double, double,
                                 cudaStream_t);

// ---- training data of the learned closure: box filter and downsample by f
// of the physical fields P(n, z, y, x) (Lu fields): block means of u_a,
// T, the velocity products u_a u_b (rhs.f's order) and u_a T, written as
// out(X, Y, Z, m) with X = Nx/f fastest, m = 0..Lu+Lr-1.
template <typename T>
__global__ void k_box_filter(const T* __restrict__ ph, int lu, int nx, int ny, int nz, int f, double* __restrict__ out) {
  const int cx = nx / f, cy = ny / f, cz = nz / f;
  const long long nc = (long long)cx * cy * cz, np = (long long)nx * ny * nz;
  const int lr = lu == 4 ? 9 : 6;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nc; e += (long long)gridDim.x * blockDim.x) {
    const int X = (int)(e % cx), Y = (int)((e / cx) % cy), Z = (int)(e / ((long long)cx * cy));
    double acc[13];
#pragma unroll
    for (int m = 0; m < 13; ++m) acc[m] = 0.0;
    for (int k = 0; k < f; ++k)
      for (int j = 0; j < f; ++j)
        for (int i = 0; i < f; ++i) {
          const long long p = ((long long)(Z * f + k) * ny + (Y * f + j)) * nx + (X * f + i);
          const double u = ph[p], v = ph[np + p], w = ph[2 * np + p];
          const double t = lu == 4 ? (double)ph[3 * np + p] : 0.0;
          acc[0] += u; acc[1] += v; acc[2] += w; acc[3] += t;
          acc[4] += u * u; acc[5] += u * v; acc[6] += v * v; acc[7] += u * w; acc[8] += v * w; acc[9] += w * w;
          acc[10] += u * t; acc[11] += v * t; acc[12] += w * t;
        }
    const double inv = 1.0 / ((double)f * f * f);
    int m = 0;
    for (int q = 0; q < lu; ++q) out[(long long)(m++) * nc + e] = acc[q] * inv;
    for (int q = 0; q < lr; ++q) out[(long long)(m++) * nc + e] = acc[4 + q] * inv;
  }
}

template <typename T>
__global__ void k_to_double(const T* __restrict__ a, double* __restrict__ b, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    b[e] = (double)a[e];
}

template <typename T>
void les_box_filter(const T* ph, int lu, int nx, int ny, int nz, int f, double* out, cudaStream_t s) {
  const long long nc = (long long)(nx / f) * (ny / f) * (nz / f);
  k_box_filter<T><<<grid_of(nc), kThreads, 0, s>>>(ph, lu, nx, ny, nz, f, out);
}
template <typename T>
void les_to_double(const T* a, double* b, long long n, cudaStream_t s) {
  k_to_double<T><<<grid_of(n), kThreads, 0, s>>>(a, b, n);
}
template void les_box_filter<double>(const double*, int, int, int, int, int, double*, cudaStream_t);
template void les_box_filter<float>(const float*, int, int, int, int, int, double*, cudaStream_t);
template void les_to_double<double>(const double*, double*, long long, cudaStream_t);
template void les_to_double<float>(const float*, double*, long long, cudaStream_t);

void les_get_mean(double2* col, int mz, int kz, int nz, int i_remove, const FftPlan* dplan, const double2* tw,
                  const FftPlan& hplan, double* u_mean, double* jump, cudaStream_t s) {
  const int ld = line_stride(nz);
  const size_t sm = sizeof(double2) * ((size_t)hplan.tw_total + (size_t)ld) + 16;
  k_get_mean<<<1, kThreads, sm, s>>>(col, mz, kz, nz, i_remove, dplan, tw, u_mean, jump);
}

}  // namespace samgpu
