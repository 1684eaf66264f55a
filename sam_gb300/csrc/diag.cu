// Diagnostics on the resident wave-space state, in FP64 whatever the working
// precision: shell spectra (spectra.f:13-90), divergence (div_check.f:11-36),
// cut-off shell energy (cl_energy.f:8-43); and the plane derivatives of the
// output path (x_deriv.f:7-25, y_deriv.f:7-28).
#include <cuda_runtime.h>
#include <math.h>

#include "common.cuh"
#include "diag.cuh"

namespace samgpu {

DiagArgs diag_args(const Grid& g, int lm, int nx2, int k_cl, double vis, int i_les, double e_cl, int precision) {
  DiagArgs d{};
  d.g = g; d.lm = lm; d.nx2 = nx2; d.k_cl = k_cl; d.vis = vis; d.i_les = i_les; d.e_cl = e_cl;
  d.precision = precision;
  return d;
}

template <typename T>
__device__ __forceinline__ void ld_c(const void* base, long long idx, double& re, double& im) {
  const cx_t<T> v = reinterpret_cast<const cx_t<T>*>(base)[idx];
  re = (double)v.x;
  im = (double)v.y;
}

// One CTA per kx plane: shell sums of this plane into partial[plane][5][lm]
// plus the divergence sum and max into div[plane][2].
template <typename T>
__global__ void k_spectra(DiagArgs d, const void* u, const void* r, double* partial, double* divp) {
  extern __shared__ double sh[];
  const Grid& g = d.g;
  const int lm = d.lm;
  double* hist = sh;               // 5 * lm
  double* red = sh + 5 * lm;       // 2 * blockDim
  for (int e = threadIdx.x; e < 5 * lm; e += blockDim.x) hist[e] = 0.0;
  __syncthreads();
  const int i = blockIdx.x;
  const long long nm = (long long)g.mx * g.my * g.mz;
  const double factor = (i == 0 || i == d.nx2) ? 1.0 : 2.0;
  const double rkx = g.wave_x * i;
  const double fac_cl = d.i_les ? sqrt(2.0 * d.e_cl / (double)d.k_cl) : 0.0;
  double dsum = 0.0, dmax = 0.0;
  for (int e = threadIdx.x; e < g.my * g.mz; e += blockDim.x) {
    const int k = e % g.mz, j = e / g.mz;
    const int iy = kwave(j, g.ky, g.my), iz = kwave(k, g.kz, g.mz);
    const int k_sq = i * i + iy * iy + iz * iz;
    const double k_mag = sqrt((double)k_sq);
    const int is = (int)(k_mag + 0.5);
    const double rky = g.wave_y * iy, rkz = g.wave_z * iz;
    const double rk_sq = rkx * rkx + rky * rky + rkz * rkz;
    double vist = 0.0;
    if (!(k_sq == 0 || d.i_les == 0)) vist = fac_cl * (0.145 + 5.01 * exp(-(3.03 * d.k_cl) / k_mag));
    const long long idx = ((long long)i * g.my + j) * g.mz + k;
    double ur[3], ui[3], rr[3], ri[3];
    for (int n = 0; n < 3; ++n) {
      ld_c<T>(u, n * nm + idx, ur[n], ui[n]);
      ld_c<T>(r, n * nm + idx, rr[n], ri[n]);
    }
    const double u_sq = ur[0] * ur[0] + ui[0] * ui[0] + ur[1] * ur[1] + ui[1] * ui[1] + ur[2] * ur[2] + ui[2] * ui[2];
    const double udu = rr[0] * ur[0] + ri[0] * ui[0] + rr[1] * ur[1] + ri[1] * ui[1] + rr[2] * ur[2] + ri[2] * ui[2];
    atomicAdd(&hist[is], factor * u_sq);
    atomicAdd(&hist[lm + is], factor * udu);
    atomicAdd(&hist[2 * lm + is], factor * rk_sq * (d.vis + vist) * u_sq);
    atomicAdd(&hist[3 * lm + is], factor * vist);
    atomicAdd(&hist[4 * lm + is], factor);
    const double dr = rkx * ur[0] + rky * ur[1] + rkz * ur[2];
    const double di = rkx * ui[0] + rky * ui[1] + rkz * ui[2];
    const double dsq = dr * dr + di * di;
    dsum += dsq;
    dmax = fmax(dmax, dsq);
  }
  red[threadIdx.x] = dsum;
  red[blockDim.x + threadIdx.x] = dmax;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      red[threadIdx.x] += red[threadIdx.x + h];
      red[blockDim.x + threadIdx.x] = fmax(red[blockDim.x + threadIdx.x], red[blockDim.x + threadIdx.x + h]);
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < 5 * lm; e += blockDim.x) partial[(long long)blockIdx.x * 5 * lm + e] = hist[e];
  if (threadIdx.x == 0) {
    divp[2 * blockIdx.x] = red[0];
    divp[2 * blockIdx.x + 1] = red[blockDim.x];
  }
}

__global__ void k_spectra_finish(DiagArgs d, const double* partial, const double* divp, double* out) {
  const int lm = d.lm, np = d.g.mx;
  for (int e = threadIdx.x; e < 5 * lm; e += blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < np; ++b) s += partial[(long long)b * 5 * lm + e];
    out[e] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ek = 0.0, ds = 0.0, dm = 0.0;
    for (int s = 0; s < lm; ++s) ek += out[s];
    for (int b = 0; b < np; ++b) { ds += divp[2 * b]; dm = fmax(dm, divp[2 * b + 1]); }
    out[5 * lm] = 0.5 * ek;
    out[5 * lm + 1] = sqrt(ds);
    out[5 * lm + 2] = sqrt(dm);
  }
}

// div_check: per kx plane sums of |div|, |div|^2, max and count > 1e-20.
template <typename T>
__global__ void k_div(DiagArgs d, const void* u, double* part) {
  __shared__ double red[4][kThreads];
  const Grid& g = d.g;
  const int i = blockIdx.x;
  const long long nm = (long long)g.mx * g.my * g.mz;
  const double rkx = g.wave_x * i;
  double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  for (int e = threadIdx.x; e < g.my * g.mz; e += blockDim.x) {
    const int k = e % g.mz, j = e / g.mz;
    const double rky = g.wave_y * kwave(j, g.ky, g.my), rkz = g.wave_z * kwave(k, g.kz, g.mz);
    const long long idx = ((long long)i * g.my + j) * g.mz + k;
    double ur[3], ui[3];
    for (int n = 0; n < 3; ++n) ld_c<T>(u, n * nm + idx, ur[n], ui[n]);
    const double dr = rkx * ur[0] + rky * ur[1] + rkz * ur[2];
    const double di = rkx * ui[0] + rky * ui[1] + rkz * ui[2];
    const double dsq = dr * dr + di * di;
    s0 += sqrt(dsq);
    s1 += dsq;
    s2 = fmax(s2, dsq);
    if (dsq > 1.e-20) s3 += 1.0;
  }
  red[0][threadIdx.x] = s0; red[1][threadIdx.x] = s1; red[2][threadIdx.x] = s2; red[3][threadIdx.x] = s3;
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
  if (threadIdx.x < 4) part[4 * blockIdx.x + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void k_div_finish(const double* part, int np, double* out) {
  if (threadIdx.x == 0) {
    double a = 0, b = 0, m = 0, n = 0;
    for (int p = 0; p < np; ++p) { a += part[4 * p]; b += part[4 * p + 1]; m = fmax(m, part[4 * p + 2]); n += part[4 * p + 3]; }
    out[0] = a; out[1] = sqrt(b); out[2] = sqrt(m); out[3] = n;
  }
}

// cl_energy: per kx plane, the reference's k_start..k_stop band of each
// (kx, ky) column and its mirror row (rows beyond Nz_min read as zero).
template <typename T>
__global__ void k_cl(DiagArgs d, const void* u, double* part) {
  __shared__ double red[kThreads];
  const Grid& g = d.g;
  const int i = blockIdx.x;
  const long long nm = (long long)g.mx * g.my * g.mz;
  const double factor = (i == 0 || i == g.nx / 2) ? 1.0 : 2.0;
  const double cs = ((double)d.k_cl - 0.5) * ((double)d.k_cl - 0.5);
  const double ce = ((double)d.k_cl + 0.5) * ((double)d.k_cl + 0.5);
  double s = 0.0;
  for (int j = threadIdx.x; j < g.my; j += blockDim.x) {
    const int iy = kwave(j, g.ky, g.my);
    const int k_sq2 = i * i + iy * iy;
    const int k_start = k_sq2 > cs ? 1 : (int)sqrt(cs - k_sq2) + 2;
    const int k_stop = k_sq2 > ce ? 0 : (int)sqrt(ce - k_sq2) + 1;
    for (int k1 = k_start; k1 <= k_stop; ++k1) {
      const int k = k1 - 1, kk = g.mz + 1 - k1;
      double s1 = 0.0, s2 = 0.0;
      for (int n = 0; n < 3; ++n) {
        double ar = 0, ai = 0, br = 0, bi = 0;
        if (k >= 0 && k < g.mz) ld_c<T>(u, n * nm + ((long long)i * g.my + j) * g.mz + k, ar, ai);
        if (kk >= 0 && kk < g.mz) ld_c<T>(u, n * nm + ((long long)i * g.my + j) * g.mz + kk, br, bi);
        s1 += ar * ar + ai * ai;
        s2 += br * br + bi * bi;
      }
      s += factor * (s1 + s2);
    }
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_sum_finish(const double* part, int np, double* out) {
  if (threadIdx.x == 0) {
    double a = 0;
    for (int p = 0; p < np; ++p) a += part[p];
    out[0] = a;
  }
}

// Spectral derivative of a real (Nx, Ny) plane along x (dir 0) or y (dir 1).
// Two real lines share one complex transform; kx (or ky) <= k_max keep i k,
// everything else (the mean and the truncated band) is zeroed.
__global__ void k_deriv(Grid g, int dir, const FftPlan* __restrict__ gpl, const double2* __restrict__ gtw,
                        const double* __restrict__ u, double* __restrict__ du, int pairs_per_cta) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ FftPlan pl;
  load_plan(&pl, gpl);
  __syncthreads();
  const int n = pl.n;
  const int ld = line_stride(n);
  double2* s_tw = reinterpret_cast<double2*>(smem_raw);
  double2* s_ln = s_tw + pl.tw_total;
  for (int e = threadIdx.x; e < pl.tw_total; e += blockDim.x) s_tw[e] = gtw[e];
  const int nrows = dir == 0 ? g.ny : g.nx;  // lines along the derivative direction
  const long long sline = dir == 0 ? g.nx : 1;
  const long long selem = dir == 0 ? 1 : g.nx;
  const int kmax = dir == 0 ? g.kx : g.ky;
  const double wave = dir == 0 ? g.wave_x : g.wave_y;
  const double ninv = 1.0 / (double)n;
  const int p0 = blockIdx.x * pairs_per_cta;
  const int np = min(pairs_per_cta, (nrows + 1) / 2 - p0);
  for (int e = threadIdx.x; e < np * n; e += blockDim.x) {
    const int L = e / n, x = e - L * n;
    const int ra = 2 * (p0 + L), rb = ra + 1;
    const double a = u[ra * sline + x * selem] * ninv;
    const double b = rb < nrows ? u[rb * sline + x * selem] * ninv : 0.0;
    s_ln[L * ld + sidx(x)] = make_double2(a, b);
  }
  __syncthreads();
  fft_lines<-1>(s_ln, ld, np, s_tw, pl);
  __syncthreads();
  // split, multiply by i k, recombine: Z'_k = i k (X_k + i Y_k) for 0 < k <= kmax,
  // conj-symmetric partner at n - k, zero elsewhere
  for (int e = threadIdx.x; e < np * (n / 2 + 1); e += blockDim.x) {
    const int L = e / (n / 2 + 1), k = e - L * (n / 2 + 1);
    double2* ln = s_ln + L * ld;
    const int kk = (n - k) % n;
    const double2 z1 = ln[sidx(k)], z2 = ln[sidx(kk)];
    double2 o1 = make_double2(0.0, 0.0), o2 = make_double2(0.0, 0.0);
    if (k >= 1 && k <= kmax) {
      // X = (z1 + conj z2)/2, Y = (z1 - conj z2)/(2i)
      const double xr = 0.5 * (z1.x + z2.x), xi = 0.5 * (z1.y - z2.y);
      const double yr = 0.5 * (z1.y + z2.y), yi = 0.5 * (z2.x - z1.x);
      const double rk = wave * k;
      const double dxr = -rk * xi, dxi = rk * xr;  // i k X
      const double dyr = -rk * yi, dyi = rk * yr;  // i k Y
      // Z'_k = dX + i dY ; Z'_{n-k} = conj(dX) + i conj(dY)
      o1 = make_double2(dxr - dyi, dxi + dyr);
      o2 = make_double2(dxr + dyi, dyr - dxi);
    }
    ln[sidx(k)] = o1;
    if (k != kk) ln[sidx(kk)] = o2;
  }
  __syncthreads();
  fft_lines<+1>(s_ln, ld, np, s_tw, pl);
  __syncthreads();
  for (int e = threadIdx.x; e < np * n; e += blockDim.x) {
    const int L = e / n, x = e - L * n;
    const int ra = 2 * (p0 + L), rb = ra + 1;
    const double2 v = s_ln[L * ld + sidx(x)];
    du[ra * sline + x * selem] = v.x;
    if (rb < nrows) du[rb * sline + x * selem] = v.y;
  }
}

// force.f:12-63: shells 1..k_force+1 (1-based) keep the energy ek0 they had
// initially.  The forced modes lie in the box |kx|,|ky|,|kz| <= k_force, which
// one thread visits in the reference's loop order (kx, then ky, then kz in
// storage order), so the shell sums are summed as force.f sums them.
template <typename T>
__global__ void k_force_shells(DiagArgs d, void* uv, const double* __restrict__ ek0, int k_force) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  using C = cx_t<T>;
  C* u = reinterpret_cast<C*>(uv);
  const Grid& g = d.g;
  const long long nm = (long long)g.mx * g.my * g.mz;
  double work[64], fac[64];
  const int ns = k_force + 1;
  for (int s = 0; s < ns; ++s) work[s] = 0.0;
  const int ix_end = min(k_force, g.mx - 1);
  for (int i = 0; i <= ix_end; ++i) {
    const double factor = (i == 0 || i == d.nx2) ? 1.0 : 2.0;
    for (int j = 0; j < g.my; ++j) {
      const int iy = kwave(j, g.ky, g.my);
      if (iy > k_force || iy < -k_force) continue;
      for (int k = 0; k < g.mz; ++k) {
        const int iz = kwave(k, g.kz, g.mz);
        if (iz > k_force || iz < -k_force) continue;
        const int is = (int)(sqrt((double)(i * i + iy * iy + iz * iz)) + 0.5);
        if (is > k_force) continue;
        const long long e = ((long long)i * g.my + j) * g.mz + k;
        double usq = 0.0;
        for (int n = 0; n < 3; ++n) {
          const C v = u[n * nm + e];
          usq += (double)v.x * (double)v.x + (double)v.y * (double)v.y;
        }
        work[is] += factor * usq;
      }
    }
  }
  fac[0] = 1.0;
  for (int s = 1; s < ns; ++s) fac[s] = sqrt(ek0[s] / work[s]);
  for (int i = 0; i <= ix_end; ++i)
    for (int j = 0; j < g.my; ++j) {
      const int iy = kwave(j, g.ky, g.my);
      if (iy > k_force || iy < -k_force) continue;
      for (int k = 0; k < g.mz; ++k) {
        const int iz = kwave(k, g.kz, g.mz);
        if (iz > k_force || iz < -k_force) continue;
        const int is = (int)(sqrt((double)(i * i + iy * iy + iz * iz)) + 0.5);
        if (is > k_force) continue;
        const long long e = ((long long)i * g.my + j) * g.mz + k;
        for (int n = 0; n < 3; ++n) {
          C v = u[n * nm + e];
          v.x = (T)((double)v.x * fac[is]);
          v.y = (T)((double)v.y * fac[is]);
          u[n * nm + e] = v;
        }
      }
    }
}

void diag_force(const DiagArgs& d, void* u, const double* ek0_dev, int k_force, cudaStream_t s) {
  if (d.precision == 32) k_force_shells<float><<<1, 32, 0, s>>>(d, u, ek0_dev, k_force);
  else k_force_shells<double><<<1, 32, 0, s>>>(d, u, ek0_dev, k_force);
}

// FP64 FMA throughput probe: 8 independent dependency chains per thread.
__global__ void k_dfma(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
         x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

double diag_fp64_peak(cudaStream_t s) {
  const int blocks = sm_count() * 2, threads = 256, iters = 20000;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return 0.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dfma<<<blocks, threads, 0, s>>>(out, iters / 10, 0.999999, 1e-7);
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0, s);
    k_dfma<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
}

void diag_set_smem_limits() {
  cudaFuncSetAttribute(k_deriv, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  cudaFuncSetAttribute(k_spectra<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  cudaFuncSetAttribute(k_spectra<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}

void diag_spectra(const DiagArgs& d, const void* u, const void* r, double* scratch, double* host_out, cudaStream_t s) {
  const int lm = d.lm;
  double* partial = scratch;
  double* divp = partial + (size_t)d.g.mx * 5 * lm;
  double* out = divp + 2 * d.g.mx;
  const size_t sm = sizeof(double) * (5 * lm + 2 * kThreads);
  if (d.precision == 32) k_spectra<float><<<d.g.mx, kThreads, sm, s>>>(d, u, r, partial, divp);
  else k_spectra<double><<<d.g.mx, kThreads, sm, s>>>(d, u, r, partial, divp);
  k_spectra_finish<<<1, kThreads, 0, s>>>(d, partial, divp, out);
  cudaMemcpyAsync(host_out, out, sizeof(double) * (5 * lm + 3), cudaMemcpyDeviceToHost, s);
}

void diag_div_check(const DiagArgs& d, const void* u, double* scratch, double* host_out, cudaStream_t s) {
  double* part = scratch;
  double* out = part + 4 * d.g.mx;
  if (d.precision == 32) k_div<float><<<d.g.mx, kThreads, 0, s>>>(d, u, part);
  else k_div<double><<<d.g.mx, kThreads, 0, s>>>(d, u, part);
  k_div_finish<<<1, 32, 0, s>>>(part, d.g.mx, out);
  cudaMemcpyAsync(host_out, out, sizeof(double) * 4, cudaMemcpyDeviceToHost, s);
}

void diag_cl_energy(const DiagArgs& d, const void* u, double* scratch, double* host_out, cudaStream_t s) {
  double* part = scratch;
  double* out = part + d.g.mx;
  if (d.precision == 32) k_cl<float><<<d.g.mx, kThreads, 0, s>>>(d, u, part);
  else k_cl<double><<<d.g.mx, kThreads, 0, s>>>(d, u, part);
  k_sum_finish<<<1, 32, 0, s>>>(part, d.g.mx, out);
  cudaMemcpyAsync(host_out, out, sizeof(double), cudaMemcpyDeviceToHost, s);
}

void diag_deriv(const Grid& g, int dir, const FftPlan* dplan, const double2* tw, const FftPlan& hplan, const double* u,
                double* du, cudaStream_t s) {
  const int n = hplan.n;
  const int ld = line_stride(n);
  const int nrows = dir == 0 ? g.ny : g.nx;
  const int pairs = (nrows + 1) / 2;
  int per = 8;
  while (per > 1 && sizeof(double2) * ((size_t)hplan.tw_total + (size_t)per * ld) > 200 * 1024) per /= 2;
  const size_t sm = sizeof(double2) * ((size_t)hplan.tw_total + (size_t)per * ld) + 16;
  const int grid = (pairs + per - 1) / per;
  k_deriv<<<grid, kThreads, sm, s>>>(g, dir, dplan, tw, u, du, per);
}

}  // namespace samgpu
