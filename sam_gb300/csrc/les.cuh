// Subgrid-model routines and get_mean (les.cu).
#pragma once
#include "common.cuh"

namespace samgpu {
void les_filter(const double* f_bar, double* f_hat, int nx, int ny, int n_var, cudaStream_t s);
// ub: 3*Nx*Ny*Nz doubles of workspace
void les_sm(const double* u, double* ub, double* vt, int nx, int ny, int nz, double c_delta_sq, double dxi, double dyi,
            double dzi, cudaStream_t s);
int les_dm_blocks(int nx, int ny, int nz);
// ub: 3*N, q: 19*N doubles (N = Nx*Ny*Nz); part: 2*les_dm_blocks; cds: 1
void les_dm(const double* u, double* ub, double* q, double* part, double* cds, double* vt, int nx, int ny, int nz,
            double alpha_sq, double dxi, double dyi, double dzi, cudaStream_t s);
// dm.f's volume-averaged C delta^2 of the physical velocity phys
// (3 fields (n, z, y, x)), clipped at zero, into cds[0]; work holds
// les_dynamic_work doubles
size_t les_dynamic_work(int nx, int ny, int nz);
template <typename T>
void les_dynamic(const T* phys, double* work, double* cds, int nx, int ny, int nz, double dxi, double dyi,
                 double dzi, cudaStream_t s);
// box filter and downsample by f (training data of the learned closure)
template <typename T>
void les_box_filter(const T* ph, int lu, int nx, int ny, int nz, int f, double* out, cudaStream_t s);
template <typename T>
void les_to_double(const T* a, double* b, long long n, cudaStream_t s);
void les_get_mean(double2* col, int mz, int kz, int nz, int i_remove, const FftPlan* dplan, const double2* tw,
                  const FftPlan& hplan, double* u_mean, double* jump, cudaStream_t s);
}  // namespace samgpu
