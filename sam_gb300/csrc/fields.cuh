// Initial fields and precision conversion (fields.cu).
#pragma once
#include <stdint.h>

#include "common.cuh"

namespace samgpu {
void fields_zero(double2* u, long long n, cudaStream_t s);
void fields_init_tg(double2* u, const Grid& g, cudaStream_t s);
void fields_init_random(double2* u, const Grid& g, uint64_t seed, int kind_u, double flct_u, int kind_t, double flct_t,
                        cudaStream_t s);
void fields_init_packet(double2* u, const Grid& g, uint64_t seed, int kx0, int ky0, int kz0, double sigma,
                        double amplitude, double noise, double xl, double yl, double zl, double buoy_fac_z,
                        double lapse, cudaStream_t s);
// Ornstein-Uhlenbeck forcing of the modes 0 < |k| <= k_f (device resident).
constexpr int kOuModesMax = 128;
struct OuForcing {
  int n_modes;
  int pad;
  long long step;
  unsigned long long seed;
  double sigma, t_l;
  int kx[kOuModesMax], ky[kOuModesMax], kz[kOuModesMax];
  double2 a[kOuModesMax][3];
};
// fills the mode list of f; returns the count, -1 when above kOuModesMax
int ou_modes(const Grid& g, double k_f, OuForcing& f);
// a = sigma xi(step 0), step = 0
void ou_init(OuForcing* dev, cudaStream_t s);
// u += dt P(k) a on the three velocity fields, then a advances one step
template <typename T> void ou_apply(cx_t<T>* u, const Grid& g, OuForcing* dev, const DevState* st, cudaStream_t s);
template <typename T> void convert_in(const double2* src, cx_t<T>* dst, long long n, cudaStream_t s);
template <typename T> void convert_out(const cx_t<T>* src, double2* dst, long long n, cudaStream_t s);
}  // namespace samgpu
