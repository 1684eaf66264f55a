// Argument blocks and launchers of the transform passes (passes_impl.cuh,
// instantiated in passes.cu, passes_f32.cu and passes_dd_*.cu).
// Strides are in complex (or real, for physical arrays) elements.
#pragma once
#include "common.cuh"

namespace samgpu {

template <typename T>
struct ZInvArgs {
  Grid g;
  // FFT schedule of length-256 lines: 0 the 16 x 16 register path, 1 the
  // compile-time Stockham stages (radix 8, 8, 4); chosen by the autotuner
  int sched;
  const cx_t<T>* in;   // rows of Nz_min modes
  cx_t<T>* out;        // A(n, z, kx, ky)
  const cx_t<T>* tw;   // twiddles of the Nz plan
  int nvar, ty, ld;
  // derive = 1: fields n >= Lu of the launch are the subgrid gradient fields
  // m = n - Lu formed from the velocity (and T) rows while loading: S_ab for
  // the six velocity products, dT/dx_a for the three buoyancy products
  int derive;
  long long in_ky, in_kx, in_n;
  long long out_kx, out_z, out_n;
};

template <typename T>
struct YInvArgs {
  Grid g;
  // FFT schedule of length-256 lines: 0 the 16 x 16 register path, 1 the
  // compile-time Stockham stages (radix 8, 8, 4); chosen by the autotuner
  int sched;
  const cx_t<T>* in;  // rows (one per kx) of Ny_min modes or Ny values
  cx_t<T>* out;       // B(n, z, y, kx)
  const cx_t<T>* tw;
  int nvar, tx, ld, in_full;
  long long in_kx, in_z, in_n;
  long long out_y, out_z, out_n;
};

// Threads of an x pass CTA.  In the FP32 16 x 16 register path (n = 256) a
// team of 16 threads transforms one line, and an 8-row tile holds 4 x 4
// input and 9 x 4 product lines: 18 teams do them in one and two full rounds
// (16 teams would need a third round a quarter full).  Other forms keep
// kThreads.
__host__ __device__ constexpr int x_threads(int bytes, bool reg16) { return bytes == 4 && reg16 ? 288 : kThreads; }

template <typename T>
struct XPassArgs {
  Grid g;
  // FFT schedule of length-256 lines: 0 the 16 x 16 register path, 1 the
  // compile-time Stockham stages (radix 8, 8, 4); chosen by the autotuner
  int sched;
  const cx_t<T>* in;   // in_mode 0: B(n, z, y, kx)
  const T* in_phys;    // in_mode 1: P(n, z, y, x)
  cx_t<T>* out;        // out_mode 1/2: C(m, z, kx, y)
  T* out_phys;         // out_mode 0: P(n, z, y, x)
  double* partials;    // vel_max partials (nblocks, lu, 4) or null
  const cx_t<T>* tw;
  // group: product lines transformed per round of out_mode 2 (a multiple of
  // the CTA's teams where it exceeds them), any split of the Lr * Y/2 lines
  int in_mode, out_mode, nin, yt, group, ld;
  // vel_max partials: max_only = 1 leaves the sums to k_parseval (FP32 form)
  int max_only;
  int* vmax;  // max_only: per-field max |u| (float bit patterns) and the NaN flag, atomically
  T fn;  // 1/(2 Nx Ny): xy_trans_f.f:20's scale and the 1/2 of the pair split (launcher)
  // subgrid stress (les = 1): input fields Lu .. Lu+Lr-1 are the gradient
  // fields of the products; nu_t = C delta^2 |S| with C delta^2 read from
  // les_cds, kappa_t = nu_t * les_prt_inv
  // les = 2: per-point coefficients les_coef[(z Ny + y) Nx + x] =
  // (C_nu, C_kappa) of the learned closure, nu_t = C_nu les_dsq |S|,
  // kappa_t = C_kappa les_dsq |S|
  int les;
  const double* les_cds;
  double les_prt_inv;
  const float2* les_coef;
  double les_dsq;
  // out_mode 4: the closure's 12 invariants of point (z Ny + y) Nx + x as
  // BF16 [16] (columns 12..14 = 1.0, the network's bias inputs; 15 = 0)
  // from the input fields S (6), dT/dx (3, when Lr = 9) and w (3);
  // f_bz = buoy_fac_z, f_n2 = N^2, f_dsq = delta^2, f_nu = viscosity
  void* feat;
  double f_bz, f_n2, f_dsq, f_nu;
  long long in_y, in_z, in_n;
  long long out_kx, out_z, out_n;
  long long out_py, out_pz, out_pn;
  FastDiv fd_mx, fd_yp, fd_nx, fd_y;  // filled by the launcher
};

template <typename T>
struct YFwdArgs {
  Grid g;
  // FFT schedule of length-256 lines: 0 the 16 x 16 register path, 1 the
  // compile-time Stockham stages (radix 8, 8, 4); chosen by the autotuner
  int sched;
  const cx_t<T>* in;  // C(m, z, kx, y)
  cx_t<T>* out;       // D(m, kx, ky, z)
  const cx_t<T>* tw;
  int nvar, tz, ld;
  long long in_kx, in_z, in_n;
  long long out_ky, out_kx, out_n;
};

template <typename T>
struct ZFwdArgs {
  Grid g;
  // FFT schedule of length-256 lines: 0 the 16 x 16 register path, 1 the
  // compile-time Stockham stages (radix 8, 8, 4); chosen by the autotuner
  int sched;
  cx_t<T>* in;  // D(m, kx, ky, z); mode 0 writes the result back here
  const cx_t<T>* tw;
  int mode, nf, ty, ld;
  long long in_ky, in_kx, in_n;
  // mode 1 (rhs): r out and u_sav in
  cx_t<T>* r;
  long long r_ky, r_kx, r_n;
  const cx_t<T>* usav;
  long long sav_ky, sav_kx, sav_n;
  // mode 2 (stage): u, r (same layout), p, device state
  cx_t<T>* u;
  cx_t<T>* p;
  long long u_ky, u_kx, u_n;
  DevState* state;
  StageConsts sc;
  // double-float form, mode 2: the integrating factor exp(-nu k^2 dt_fac)
  // as products of per-direction tables [2][Mx + My + Mz] (velocity, then
  // temperature with nu / Pr), written by launch_if_tables for this stage
  const dd* ift;
  T nz_inv;                  // filled by the launcher: 1/Nz
  FastDiv fd_t, fd_m;  // filled by the launcher: ty, Nz_min
};

template <typename T> void launch_z_inv(const ZInvArgs<T>& a, const FftPlan* pl, size_t smem, cudaStream_t s);
template <typename T> void launch_y_inv(const YInvArgs<T>& a, const FftPlan* pl, size_t smem, cudaStream_t s);
template <typename T> void launch_x_pass(const XPassArgs<T>& a, const FftPlan* pl, size_t smem, cudaStream_t s);
template <typename T> int x_pass_blocks(const XPassArgs<T>& a);
template <typename T> void launch_y_fwd(const YFwdArgs<T>& a, const FftPlan* pl, size_t smem, cudaStream_t s);
template <typename T> void launch_z_fwd(const ZFwdArgs<T>& a, const FftPlan* pl, size_t smem, cudaStream_t s);
template <typename T> void smem_limits_zinv(int optin);
template <typename T> void smem_limits_yinv(int optin);
template <typename T> void smem_limits_x(int optin);
template <typename T> void smem_limits_yfwd(int optin);
template <typename T> void smem_limits_zfwd(int optin);
// every pass of precision T opted into the device's largest dynamic shared memory
template <typename T> inline void set_smem_limits() {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  smem_limits_zinv<T>(optin);
  smem_limits_yinv<T>(optin);
  smem_limits_x<T>(optin);
  smem_limits_yfwd<T>(optin);
  smem_limits_zfwd<T>(optin);
}
// vmax (max_only forms): ints 0..7 hold the per-field maxima (FP32 form: the
// float bit patterns in ints 0..3; double-float form: 64-bit keys of
// dd_abs_key in ints 0..7, vkind = 1), int 8 the non-finite flag
void launch_vel_max_finish(const double* partials, int nblk, const Grid& g, DevState* st, int i_cfl, double cfl0,
                           double adv_cfl_limit, cudaStream_t s, const double* pv = nullptr, int npv = 0,
                           int* vmax = nullptr, int vkind = 0);
// The double-float form's integrating-factor tables of one stage (mode-2
// z forward): t[w * (Mx + My + Mz) + r] = exp(-nu_w dt_fac k_r^2) for the
// wave numbers of kx (r < Mx), ky, then kz, with nu_0 = vis and nu_1 =
// vis / Pr, dt_fac = (gamma + zeta) dt (sam.f:293-297), dt read on the device.
void launch_if_tables(const DevState* st, const StageConsts& sc, const Grid& g, dd* t, cudaStream_t s);
constexpr int kVmaxInts = 16;  // the vmax block at the end of pv
// vel_max's sums from wave space (Parseval), FP64 arithmetic on the state U
// (Lu fields (kx, ky, kz)): pv[b * Lu + f] = block b's share of
// sum w |u|^2 (w = 1 for kx = 0, 2 otherwise), pv[npv * Lu + f] = u(0,0,0).
constexpr int kParsevalBlocks = 152 * 4;
template <typename T> void launch_parseval(const cx_t<T>* u, const Grid& g, double* pv, cudaStream_t s);
void launch_x2z(const double2* in, double2* out, const Grid& g, int nvar, int nx2, cudaStream_t s);

}  // namespace samgpu
