// Planes output path (planes.cu): the wave-space fields of sam.f:145-166 and
// the plane extraction of write_planes.f.
#pragma once
#include "common.cuh"

namespace samgpu {

constexpr int kPlaneFieldsMax = 16;  // 2 Lu + 2 (Lu - 1) <= 14
constexpr int kPlanesMax = 16;       // planes of each orientation per call

// Field f of the planes batch is op[f] applied to src[f] (a field of u, or
// -1 for the pressure): 0 copy, 1 i kz, 2 i ky, 3 i kx (with the wave factors).
struct PlaneFields {
  int nf;
  int src[kPlaneFieldsMax];
  int op[kPlaneFieldsMax];
};

// Plane selection (0-based indices) and, per output slot, the batch field it
// reads: xy slots read fxy[s], xz slots fxz[s], yz slots fyz[s].
struct PlaneSel {
  int n_xy, n_xz, n_yz, n_out;
  int k_xy[kPlanesMax], j_xz[kPlanesMax], i_yz[kPlanesMax];
  int fxy[kPlaneFieldsMax], fxz[kPlaneFieldsMax], fyz[kPlaneFieldsMax];
};

// W(f, kx, ky, kz) for the batch from the resident u (lu fields) and p, both
// in the resident (field, kx, ky, kz) layout.
template <typename T>
void planes_fields(const Grid& g, const PlaneFields& pf, const cx_t<T>* u, const cx_t<T>* p, cx_t<T>* w,
                   cudaStream_t s);
// xy(Nx,Ny,n_out,n_xy), xz(Nx,Nz,n_out,n_xz), yz(Ny,Nz,n_out,n_yz) in FP64 from
// the physical batch ph(f, z, y, x).
template <typename T>
void planes_gather(const Grid& g, const PlaneSel& sel, const T* ph, double* xy, double* xz, double* yz,
                   cudaStream_t s);
}  // namespace samgpu
