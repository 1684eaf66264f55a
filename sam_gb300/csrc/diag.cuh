// Diagnostics and plane derivatives (diag.cu).
#pragma once
#include "common.cuh"

namespace samgpu {
struct DiagArgs {
  Grid g;
  int lm, nx2, k_cl, i_les, precision;
  double vis, e_cl;
};
DiagArgs diag_args(const Grid& g, int lm, int nx2, int k_cl, double vis, int i_les, double e_cl, int precision);
void diag_set_smem_limits();
// force.f on the resident state: ek0_dev holds the initial shell energies
// (spectra's ek), k_force + 1 <= 64 shells
void diag_force(const DiagArgs& d, void* u, const double* ek0_dev, int k_force, cudaStream_t s);
// measured FP64 FMA throughput of this GPU in TFLOP/s
double diag_fp64_peak(cudaStream_t s);
// scratch must hold (5*Lm+2)*Nx_min + 5*Lm + 3 doubles
void diag_spectra(const DiagArgs& d, const void* u, const void* r, double* scratch, double* host_out, cudaStream_t s);
void diag_div_check(const DiagArgs& d, const void* u, double* scratch, double* host_out, cudaStream_t s);
void diag_cl_energy(const DiagArgs& d, const void* u, double* scratch, double* host_out, cudaStream_t s);
void diag_deriv(const Grid& g, int dir, const FftPlan* dplan, const double2* tw, const FftPlan& hplan, const double* u,
                double* du, cudaStream_t s);
}  // namespace samgpu
