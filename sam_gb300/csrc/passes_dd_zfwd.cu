// The double-float instantiation of the forward z pass (passes_impl.cuh) and
// the form's integrating-factor tables.
#include "passes_impl.cuh"

namespace samgpu {

SAMGPU_INST_ZFWD(dd)

// exp(-nu (k_x^2 + k_y^2 + k_z^2) dt_fac) = e(k_x) e(k_y) e(k_z): the three
// factors in FP64 (one exp per wave number and viscosity), rounded to pairs;
// the z-forward epilogue multiplies them in double-float arithmetic.
__global__ void k_if_tables(const DevState* __restrict__ st, StageConsts sc, Grid g, dd* __restrict__ t) {
  const double dt = st->dt;
  const double vis_f = sc.vis * (sc.gamma * dt + sc.zeta * dt);  // sam.f:293-295
  const int n = g.mx + g.my + g.mz;
  for (int e = threadIdx.x; e < 2 * n; e += blockDim.x) {
    const int w = e >= n, r = e - w * n;
    double kv;
    if (r < g.mx) kv = g.wave_x * (double)r;
    else if (r < g.mx + g.my) kv = g.wave_y * (double)kwave(r - g.mx, g.ky, g.my);
    else kv = g.wave_z * (double)kwave(r - g.mx - g.my, g.kz, g.mz);
    const double v = w ? vis_f * sc.pr_inv : vis_f;  // sam.f:297
    t[e] = dd(exp(-v * kv * kv));
  }
}

void launch_if_tables(const DevState* st, const StageConsts& sc, const Grid& g, dd* t, cudaStream_t s) {
  k_if_tables<<<1, kThreads, 0, s>>>(st, sc, g, t);
}

}  // namespace samgpu
