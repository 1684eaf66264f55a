// Initial fields written straight into the resident wave-space state, and the
// FP64 <-> working-precision conversions of upload / download.
//
//  * Taylor-Green: exact wave-space coefficients of sin x cos y cos z.
//  * random solenoidal: the alpha/beta construction of initial_field.f:62-122
//    with a counter-based RNG (splitmix64, Steele, Lea & Flood 2014) so every
//    mode's phases depend only on (seed, stream, kx, ky, kz); spectra
//    kind 0 = k^2 (e_k, initial_field.f:363-365) and kind 6 = k^4 exp(-2(k/4)^2);
//    then enforce_symm (initial_field.f:422-460) and rescale (:463-497).
//  * Gaussian-enveloped internal-wave packet, set mode by mode from the
//    envelope's Fourier transform.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "common.cuh"
#include "fields.cuh"

namespace samgpu {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double uniform01(uint64_t seed, int stream, int i, int j, int k) {
  const uint64_t ctr = ((((uint64_t)stream * 4096u + (uint64_t)i) * 4096u + (uint64_t)j) * 4096u) + (uint64_t)k;
  const uint64_t x = mix64(seed ^ mix64(ctr));
  return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ double spectrum(double k, int kind) {
  if (kind == 6) return k * k * k * k * exp(-2.0 * (k / 4.0) * (k / 4.0));
  return k * k;
}

// Fields are FP64 (lu, mx, my, mz) compact; kx index i, ky index j, kz index k.
__global__ void k_init_random(double2* u, Grid g, uint64_t seed, int kind_u, int kind_t) {
  const long long nm = (long long)g.mx * g.my * g.mz;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nm; e += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(e % g.mz);
    const int j = (int)((e / g.mz) % g.my);
    const int i = (int)(e / ((long long)g.mz * g.my));
    const int ix = i, iy = kwave(j, g.ky, g.my), iz = kwave(k, g.kz, g.mz);
    const double two_pi = 6.283185307179586476925286766559;
    const double factor = 1.0 / two_pi;
    const double rkx = g.wave_x * ix, rky = g.wave_y * iy, rkz = g.wave_z * iz;
    const double rk_sq2 = rkx * rkx + rky * rky;
    const double rk12_mag = sqrt(rk_sq2);
    const double rk_mag = sqrt(rk_sq2 + rkz * rkz);
    const int k_sq = ix * ix + iy * iy + iz * iz;
    const double k_mag = sqrt((double)k_sq);
    const double k_mag1 = fmax(k_mag, 1.0e-8);
    const double f = sqrt(spectrum(k_mag, kind_u) * factor) / k_mag1;
    const double th1 = two_pi * uniform01(seed, 0, i, j, k);
    const double th2 = two_pi * uniform01(seed, 1, i, j, k);
    const double phi = two_pi * uniform01(seed, 2, i, j, k);
    const double ar = f * cos(th1) * cos(phi), ai = f * sin(th1) * cos(phi);
    const double br = f * cos(th2) * sin(phi), bi = f * sin(th2) * sin(phi);
    double2 u1, u2, u3;
    if (rk12_mag == 0.0) {
      u1 = make_double2(ar, ai);
      u2 = make_double2(br, bi);
      u3 = make_double2(0.0, 0.0);
    } else {
      const double denom = 1.0 / (rk_mag * rk12_mag);
      u1 = make_double2((ar * rk_mag * rky + br * rkx * rkz) * denom, (ai * rk_mag * rky + bi * rkx * rkz) * denom);
      u2 = make_double2((br * rky * rkz - ar * rk_mag * rkx) * denom, (bi * rky * rkz - ai * rk_mag * rkx) * denom);
      u3 = make_double2(-br * rk12_mag / rk_mag, -bi * rk12_mag / rk_mag);
    }
    u[e] = u1;
    u[nm + e] = u2;
    u[2 * nm + e] = u3;
    if (g.lu == 4) {
      const double ft = sqrt(spectrum(k_mag, kind_t) * factor) / k_mag1;
      const double th = two_pi * uniform01(seed, 3, i, j, k);
      u[3 * nm + e] = make_double2(ft * cos(th), ft * sin(th));
    }
  }
}

// enforce_symm on the kx = 0 plane of fields n0 .. n0+nvar-1; every target
// reads a source that is never itself a target, so one pass suffices.
__global__ void k_enforce_symm(double2* u, Grid g, int n0, int nvar) {
  const long long nm = (long long)g.mx * g.my * g.mz;
  const int tot = g.my * g.mz * nvar;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
    const int k = e % g.mz;
    const int j = (e / g.mz) % g.my;
    const int n = n0 + e / (g.mz * g.my);
    double2* f = u + n * nm;  // kx = 0 plane: index j*mz + k
    if (j == 0 && k == 0) {
      const double2 v = f[0];  // 0.5 * (u + conj u)
      f[0] = make_double2(0.5 * (v.x + v.x), 0.5 * (v.y - v.y));
    } else if (k == 0 && j > g.ky) {
      const double2 s = f[(g.my - j) * g.mz];
      f[j * g.mz] = make_double2(s.x, -s.y);
    } else if (j == 0 && k > g.kz) {
      const double2 s = f[g.mz - k];
      f[k] = make_double2(s.x, -s.y);
    } else if (j >= 1 && k > g.kz) {
      const double2 s = f[(g.my - j) * g.mz + (g.mz - k)];
      f[j * g.mz + k] = make_double2(s.x, -s.y);
    }
  }
}

// rescale (initial_field.f:470-494): one CTA sums |u|^2 over the stored modes
// in a fixed order, then every thread scales.
__global__ void k_rescale(double2* u, Grid g, int n0, int nvar, double flct) {
  __shared__ double red[1024];
  __shared__ double scale;
  const long long nm = (long long)g.mx * g.my * g.mz;
  double s = 0.0;
  for (long long e = threadIdx.x; e < nm * nvar; e += blockDim.x) {
    const double2 v = u[n0 * nm + e];
    s += v.x * v.x + v.y * v.y;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) scale = red[0] > 0.0 ? flct * sqrt((double)nvar) / sqrt(red[0]) : 1.0;
  __syncthreads();
  for (long long e = threadIdx.x; e < nm * nvar; e += blockDim.x) {
    double2 v = u[n0 * nm + e];
    v.x *= scale;
    v.y *= scale;
    u[n0 * nm + e] = v;
  }
}

__global__ void k_zero(double2* u, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    u[e] = make_double2(0.0, 0.0);
}

__global__ void k_init_tg(double2* u, Grid g) {
  // u = sin x cos y cos z, v = -cos x sin y cos z: kx = 1, ky = +-1, kz = +-1
  const long long nm = (long long)g.mx * g.my * g.mz;
  const int t = threadIdx.x;
  if (t < 4) {
    const int sj = (t & 1) ? 1 : -1, sk = (t & 2) ? 1 : -1;
    const int j = sj > 0 ? 1 : g.my - 1, k = sk > 0 ? 1 : g.mz - 1;
    const long long e = ((long long)1 * g.my + j) * g.mz + k;
    u[e] = make_double2(0.0, -0.125);
    u[nm + e] = make_double2(0.0, 0.125 * sj);
  }
}

__global__ void k_init_packet(double2* u, Grid g, int kx0, int ky0, int kz0, double sigma, double amplitude,
                              double vol_fac, double ex, double ey, double ez, double tfac) {
  const long long nm = (long long)g.mx * g.my * g.mz;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nm; e += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(e % g.mz);
    const int j = (int)((e / g.mz) % g.my);
    const int i = (int)(e / ((long long)g.mz * g.my));
    const int ix = i, iy = kwave(j, g.ky, g.my), iz = kwave(k, g.kz, g.mz);
    const double sgn = ((ix + iy + iz) & 1) ? -1.0 : 1.0;
    const double px = g.wave_x * (ix - kx0), py = g.wave_y * (iy - ky0), pz = g.wave_z * (iz - kz0);
    const double mxw = g.wave_x * (ix + kx0), myw = g.wave_y * (iy + ky0), mzw = g.wave_z * (iz + kz0);
    const double gm = vol_fac * sgn * exp(-0.5 * sigma * sigma * (px * px + py * py + pz * pz));
    const double gp = vol_fac * sgn * exp(-0.5 * sigma * sigma * (mxw * mxw + myw * myw + mzw * mzw));
    const double re_c = 0.5 * (gm + gp);
    const double im_c_im = -0.5 * (gm - gp);  // transform of Im(G e^{ik0.x}) is i * im_c_im
    const double rkx = g.wave_x * ix, rky = g.wave_y * iy, rkz = g.wave_z * iz;
    const double rk_sq = rkx * rkx + rky * rky + rkz * rkz;
    double a0 = amplitude * ex * re_c, a1 = amplitude * ey * re_c, a2 = amplitude * ez * re_c;
    if (rk_sq > 0.0) {
      const double dv = (rkx * a0 + rky * a1 + rkz * a2) / rk_sq;
      a0 -= rkx * dv;
      a1 -= rky * dv;
      a2 -= rkz * dv;
    } else {
      a0 = a1 = a2 = 0.0;
    }
    u[e].x += a0;
    u[nm + e].x += a1;
    u[2 * nm + e].x += a2;
    if (g.lu == 4 && tfac != 0.0) u[3 * nm + e].y += tfac * im_c_im;
  }
}

// ---- precision conversion between the FP64 staging copy and the state
template <typename T>
__global__ void k_convert_in(const double2* __restrict__ src, cx_t<T>* __restrict__ dst, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const double2 v = src[e];
    cx_t<T> o;
    o.x = (T)v.x;
    o.y = (T)v.y;
    dst[e] = o;
  }
}
template <typename T>
__global__ void k_convert_out(const cx_t<T>* __restrict__ src, double2* __restrict__ dst, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const cx_t<T> v = src[e];
    dst[e] = make_double2((double)v.x, (double)v.y);
  }
}

static int grid_for(long long n) {
  long long g = (n + kThreads - 1) / kThreads;
  if (g > sm_count() * 32) g = sm_count() * 32;
  if (g < 1) g = 1;
  return (int)g;
}

void fields_zero(double2* u, long long n, cudaStream_t s) { k_zero<<<grid_for(n), kThreads, 0, s>>>(u, n); }

void fields_init_tg(double2* u, const Grid& g, cudaStream_t s) {
  fields_zero(u, (long long)g.lu * g.mx * g.my * g.mz, s);
  k_init_tg<<<1, 32, 0, s>>>(u, g);
}

void fields_init_random(double2* u, const Grid& g, uint64_t seed, int kind_u, double flct_u, int kind_t, double flct_t,
                        cudaStream_t s) {
  const long long nm = (long long)g.mx * g.my * g.mz;
  k_init_random<<<grid_for(nm), kThreads, 0, s>>>(u, g, seed, kind_u, kind_t);
  k_enforce_symm<<<grid_for((long long)g.my * g.mz * 3), kThreads, 0, s>>>(u, g, 0, 3);
  k_rescale<<<1, 1024, 0, s>>>(u, g, 0, 3, flct_u);
  if (g.lu == 4) {
    k_enforce_symm<<<grid_for((long long)g.my * g.mz), kThreads, 0, s>>>(u, g, 3, 1);
    k_rescale<<<1, 1024, 0, s>>>(u, g, 3, 1, flct_t);
  }
}

void fields_init_packet(double2* u, const Grid& g, uint64_t seed, int kx0, int ky0, int kz0, double sigma,
                        double amplitude, double noise, double xl, double yl, double zl, double buoy_fac_z,
                        double lapse, cudaStream_t s) {
  const long long nm = (long long)g.mx * g.my * g.mz;
  if (noise > 0.0) {
    fields_init_random(u, g, seed, 0, noise, 0, 0.0, s);
    if (g.lu == 4) fields_zero(u + 3 * nm, nm, s);
  } else {
    fields_zero(u, g.lu * nm, s);
  }
  const double qx = g.wave_x * kx0, qy = g.wave_y * ky0, qz = g.wave_z * kz0;
  double ex = qz, ey = 0.0, ez = -qx;
  double en = sqrt(ex * ex + ey * ey + ez * ez);
  if (en == 0.0) { ex = 0.0; ey = 0.0; ez = 1.0; en = 1.0; }
  ex /= en; ey /= en; ez /= en;
  const double q2 = qx * qx + qy * qy + qz * qz;
  const double n2 = buoy_fac_z * lapse;
  const double omega = sqrt(n2 * (qx * qx + qy * qy) / (q2 > 0 ? q2 : 1.0));
  const double vol_fac = pow(sigma * sqrt(2.0 * 3.14159265358979323846), 3.0) / (xl * yl * zl);
  const double tfac = omega > 0.0 ? lapse * amplitude * ez / omega : 0.0;
  k_init_packet<<<grid_for(nm), kThreads, 0, s>>>(u, g, kx0, ky0, kz0, sigma, amplitude, vol_fac, ex, ey, ez, tfac);
  k_enforce_symm<<<grid_for((long long)g.my * g.mz * g.lu), kThreads, 0, s>>>(u, g, 0, g.lu);
}

template <typename T>
void convert_in(const double2* src, cx_t<T>* dst, long long n, cudaStream_t s) {
  k_convert_in<T><<<grid_for(n), kThreads, 0, s>>>(src, dst, n);
}
template <typename T>
void convert_out(const cx_t<T>* src, double2* dst, long long n, cudaStream_t s) {
  k_convert_out<T><<<grid_for(n), kThreads, 0, s>>>(src, dst, n);
}
// ------------------------------------------------ Ornstein-Uhlenbeck forcing
// Low-wavenumber stochastic forcing: every stored mode with 0 < |k| <= k_f
// (kx = 0 modes only in the half ky > 0 or ky = 0, kz > 0; their mirror images
// get the conjugate) carries three complex amplitudes a that follow an exact
// OU discretisation a <- rho a + sigma sqrt(1 - rho^2) xi, rho = exp(-dt/T_L),
// xi = (g1 + i g2)/sqrt(2) with g from Box-Muller on two splitmix64 uniforms
// keyed by (seed, step, mode, component).  After each step the velocity gets
// u += dt P(k) a (P the solenoidal projection), then a advances one step.

__device__ __forceinline__ double ou_uniform(uint64_t seed, long long step, int mode, int q) {
  const uint64_t ctr = ((uint64_t)step << 20) ^ ((uint64_t)mode << 4) ^ (uint64_t)q;
  const uint64_t x = mix64(seed ^ mix64(ctr ^ 0xA5A5A5A5A5A5A5A5ULL));
  return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ double2 ou_xi(uint64_t seed, long long step, int mode, int comp) {
  const double u1 = 1.0 - ou_uniform(seed, step, mode, 2 * comp);  // (0, 1]
  const double u2 = ou_uniform(seed, step, mode, 2 * comp + 1);
  const double rad = sqrt(-2.0 * log(u1)) * 0.70710678118654752440;
  double sn, cs;
  sincospi(2.0 * u2, &sn, &cs);
  return make_double2(rad * cs, rad * sn);
}

__global__ void k_ou_init(OuForcing* f) {
  const int m = threadIdx.x;
  if (m >= f->n_modes) return;
  for (int c = 0; c < 3; ++c) {
    const double2 xi = ou_xi(f->seed, 0, m, c);
    f->a[m][c] = make_double2(f->sigma * xi.x, f->sigma * xi.y);
  }
  if (m == 0) f->step = 0;
}

template <typename T>
__global__ void k_ou_apply(cx_t<T>* u, Grid g, OuForcing* f, const DevState* st) {
  using C = cx_t<T>;
  const int m = threadIdx.x;
  const long long step = f->step + 1;
  if (m < f->n_modes) {
    const double dt = st->dt;
    const int kx = f->kx[m], ky = f->ky[m], kz = f->kz[m];
    const double wx = g.wave_x * kx, wy = g.wave_y * ky, wz = g.wave_z * kz;
    const double k2 = wx * wx + wy * wy + wz * wz;
    double2 a[3] = {f->a[m][0], f->a[m][1], f->a[m][2]};
    const double dr = (wx * a[0].x + wy * a[1].x + wz * a[2].x) / k2;
    const double di = (wx * a[0].y + wy * a[1].y + wz * a[2].y) / k2;
    const double kv[3] = {wx, wy, wz};
    const long long nm = (long long)g.mx * g.my * g.mz;
    const int jy = ky >= 0 ? ky : ky + g.my, jz = kz >= 0 ? kz : kz + g.mz;
    const long long at = ((long long)kx * g.my + jy) * g.mz + jz;
    const long long mirror = kx == 0 ? ((long long)(ky > 0 ? g.my - ky : -ky) * g.mz + (kz > 0 ? g.mz - kz : -kz)) : -1;
    for (int c = 0; c < 3; ++c) {
      const double fr = (a[c].x - kv[c] * dr) * dt, fi = (a[c].y - kv[c] * di) * dt;
      C* p = u + c * nm + at;
      *p = mk<C>(p->x + (T)fr, p->y + (T)fi);
      if (mirror >= 0) {
        C* q = u + c * nm + mirror;
        *q = mk<C>(q->x + (T)fr, q->y - (T)fi);
      }
    }
    const double rho = exp(-dt / f->t_l);
    const double amp = f->sigma * sqrt(1.0 - rho * rho);
    for (int c = 0; c < 3; ++c) {
      const double2 xi = ou_xi(f->seed, step, m, c);
      f->a[m][c] = make_double2(rho * a[c].x + amp * xi.x, rho * a[c].y + amp * xi.y);
    }
  }
  __syncthreads();
  if (m == 0) f->step = step;
}

int ou_modes(const Grid& g, double k_f, OuForcing& f) {
  f.n_modes = 0;
  const int kk = (int)floor(k_f);
  for (int kx = 0; kx <= kk; ++kx)
    for (int ky = -kk; ky <= kk; ++ky)
      for (int kz = -kk; kz <= kk; ++kz) {
        const double k2 = (double)kx * kx + (double)ky * ky + (double)kz * kz;
        if (k2 == 0.0 || k2 > k_f * k_f) continue;
        if (kx == 0 && !(ky > 0 || (ky == 0 && kz > 0))) continue;
        if (kx > g.kx || abs(ky) > g.ky || abs(kz) > g.kz) continue;
        if (f.n_modes >= kOuModesMax) return -1;
        f.kx[f.n_modes] = kx;
        f.ky[f.n_modes] = ky;
        f.kz[f.n_modes] = kz;
        ++f.n_modes;
      }
  return f.n_modes;
}

void ou_init(OuForcing* dev, cudaStream_t s) { k_ou_init<<<1, kOuModesMax, 0, s>>>(dev); }

template <typename T>
void ou_apply(cx_t<T>* u, const Grid& g, OuForcing* dev, const DevState* st, cudaStream_t s) {
  k_ou_apply<T><<<1, kOuModesMax, 0, s>>>(u, g, dev, st);
}
template void ou_apply<float>(float2*, const Grid&, OuForcing*, const DevState*, cudaStream_t);
template void ou_apply<double>(double2*, const Grid&, OuForcing*, const DevState*, cudaStream_t);

template void convert_in<float>(const double2*, float2*, long long, cudaStream_t);
template void convert_out<float>(const float2*, double2*, long long, cudaStream_t);
template void convert_in<double>(const double2*, double2*, long long, cudaStream_t);
template void convert_out<double>(const double2*, double2*, long long, cudaStream_t);
template void convert_in<dd>(const double2*, ddc*, long long, cudaStream_t);
template void convert_out<dd>(const ddc*, double2*, long long, cudaStream_t);

}  // namespace samgpu
