/*
 * CPU oracle for the SAM pseudo-spectral RK3 step -- TEST INFRASTRUCTURE ONLY.
 *
 * FP64 restatement of the reference's periodic hot path with one MPI rank.
 * Every routine cites the reference file:line it follows.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the
 * checker; the shipped CUDA library never links it.
 *
 * Layout helpers (0-based, Fortran column-major, nxp = Nx_min, nzp = Nze):
 *   W(k,j,i,n)  wave space  (Nze, Ny_min, Nx_min, n)     sam.f:93
 *   ZB(j,i,k,n) z_trans_b   (Ny_min, Nx_min, Nze, n)     z_trans_b.f:10-13
 *   XY(j,i,k,n) x2z output  (Ny, Nx/2, Nz, n) complex    x2z_decomp.f:17
 *   P(i,j,k,n)  physical    (Nx, Ny, Nz, n) real         sam.f:94
 */
#include "sam_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "so_fft.h"

struct so_ctx {
  so_config cfg;
  int nx, ny, nz, nx2, nze;
  int kx_max, ky_max, kz_max, nx_min, ny_min, nz_min;
  int lu, lr, lm, k_cl;
  double wave_x, wave_y, wave_z, pr_inv;
  double gamma[4], zeta[4], adv_cfl_limit;
  double time, dt;
  double u_avg[4], u_var[4], u_max[4], energy, cfl_x, cfl_y, cfl_z;
  double a_cl, b_cl, c_cl;
  int *k_x, *k_y, *k_z;
  so_rplan px, pxr_y, pzr; /* rfft along x (trigx), along y (trigyr), along z (trigzr) */
  so_cplan py, pz;        /* cfft along y (trigy) and z (trigz) */
  /* stage buffers */
  so_cplx *zb;   /* z_trans_b output, also x2z temp */
  double *uu;    /* physical fields (Nx,Ny,Nz,Lr) */
  so_cplx *usav; /* (Nz_min,Ny_min,Nx_min,2) */
  /* Ornstein-Uhlenbeck forcing (so_set_forcing) */
  int ou_n;
  long long ou_step;
  uint64_t ou_seed;
  double ou_sigma, ou_tl;
  int ou_k[128][3];
  so_cplx ou_a[128][3];
  /* subgrid closure coupled into the stage (so_set_les) */
  int les_model;      /* 0 off, 1 Smagorinsky, 2 dynamic (dm.f coefficient) */
  int les_stage;      /* set by so_stage while the gradient fields are valid */
  double les_cds;     /* C delta^2 in use */
  double les_c_smag, les_prt_inv;
  so_cplx *les_w;     /* derived wave fields (Nze, Ny_min, Nx_min, Lr) */
  so_cplx *les_zb;    /* their z_trans_b blocks */
  double *les_g;      /* physical gradient fields (Nx, Ny, Nz, Lr) */
  double *les_uh;     /* haloed velocity (Lx, Ly, Lz, 3) for so_dm */
  double *les_vt;     /* haloed vt of so_dm */
  float les_mlp[5122]; /* learned closure parameters (so_mlp_set) */
  float *les_cf;      /* learned closure: (C_nu, C_kappa) per point, from stage 1 */
};

static const double SO_PI = 3.14159265358979323846;

#define W_IDX(c, k, j, i, n) \
  ((size_t)(k) + (size_t)(c)->nze * ((size_t)(j) + (size_t)(c)->ny_min * ((size_t)(i) + (size_t)(c)->nx_min * (size_t)(n))))
#define ZB_IDX(c, j, i, k, n) \
  ((size_t)(j) + (size_t)(c)->ny_min * ((size_t)(i) + (size_t)(c)->nx_min * ((size_t)(k) + (size_t)(c)->nze * (size_t)(n))))
#define XY_IDX(c, j, i, k, n) \
  ((size_t)(j) + (size_t)(c)->ny * ((size_t)(i) + (size_t)(c)->nx2 * ((size_t)(k) + (size_t)(c)->nz * (size_t)(n))))
#define P_IDX(c, i, j, k, n) \
  ((size_t)(i) + (size_t)(c)->nx * ((size_t)(j) + (size_t)(c)->ny * ((size_t)(k) + (size_t)(c)->nz * (size_t)(n))))

static void set_threads(const so_ctx *c) {
#ifdef _OPENMP
  if (c->cfg.nthreads > 0) omp_set_num_threads(c->cfg.nthreads);
#else
  (void)c;
#endif
}

/* ------------------------------------------------------------------ setup */

/* init.f:49-73 (kmax, minimal dims), init.f:117-145 (RK coefficients),
 * fft_init.f:41-78 (scales, integer wave numbers), sam.f:68-69 (Lm). */
so_ctx *so_create(const so_config *cfg) {
  if (cfg->nx < 2 || cfg->nx % 2 || cfg->ny < 1 || cfg->nz < 1) return NULL;
  so_ctx *c = (so_ctx *)calloc(1, sizeof(so_ctx));
  c->cfg = *cfg;
  c->nx = cfg->nx; c->ny = cfg->ny; c->nz = cfg->nz;
  c->nx2 = c->nx / 2;
  c->nze = c->nz; /* periodic z only (z_trans_b.f:30-52) */
  switch (cfg->n_dealias) {
    case 0:
      c->kx_max = c->nx / 2 - 1; c->ky_max = c->ny / 2 - 1; c->kz_max = c->nz / 2 - 1;
      break;
    case 2:
      c->kx_max = c->nx / 2 - 1;
      c->ky_max = (int)(((double)c->ny - 0.1) / 3.0);
      c->kz_max = (int)(((double)c->nz - 0.1) / 3.0);
      break;
    default:
      c->kx_max = (int)(((double)c->nx - 0.1) / 3.0);
      c->ky_max = (int)(((double)c->ny - 0.1) / 3.0);
      c->kz_max = (int)(((double)c->nz - 0.1) / 3.0);
  }
  if (c->ky_max < 0) c->ky_max = 0;
  if (c->kz_max < 0) c->kz_max = 0;
  c->nx_min = c->kx_max + 1;
  c->ny_min = 2 * c->ky_max + 1;
  c->nz_min = 2 * c->kz_max + 1;
  c->lu = cfg->i_strat ? 4 : 3;
  c->lr = cfg->i_strat ? 9 : 6;
  int ksq = c->kx_max * c->kx_max + c->ky_max * c->ky_max + c->kz_max * c->kz_max;
  c->lm = (int)(sqrt((double)ksq) + 0.5) + 1;
  c->k_cl = (int)(c->nx / 3.0);
  c->a_cl = 0.145; c->b_cl = 5.01; c->c_cl = 3.03;
  c->wave_x = 2.0 * SO_PI / cfg->xl;
  c->wave_y = 2.0 * SO_PI / cfg->yl;
  c->wave_z = 2.0 * SO_PI / cfg->zl;
  c->pr_inv = 1.0 / cfg->pr;
  c->k_x = (int *)malloc(sizeof(int) * (size_t)c->nx_min);
  c->k_y = (int *)malloc(sizeof(int) * (size_t)c->ny_min);
  c->k_z = (int *)malloc(sizeof(int) * (size_t)c->nz_min);
  for (int i = 0; i < c->nx_min; ++i) c->k_x[i] = i;
  for (int j = 0; j < c->ny_min; ++j) c->k_y[j] = j <= c->ky_max ? j : j - c->ny_min;
  for (int k = 0; k < c->nz_min; ++k) c->k_z[k] = k <= c->kz_max ? k : k - c->nz_min;
  for (int n = 0; n < 4; ++n) c->gamma[n] = c->zeta[n] = 0.0;
  if (cfg->nrk_max == 1) {
    c->gamma[0] = 1.0; c->adv_cfl_limit = 1.0;
  } else if (cfg->nrk_max == 2) {
    c->gamma[0] = 1.0; c->gamma[1] = 0.5; c->zeta[1] = -0.5; c->adv_cfl_limit = 1.0;
  } else {
    c->gamma[0] = 8.0 / 15.0; c->gamma[1] = 5.0 / 12.0; c->gamma[2] = 3.0 / 4.0;
    c->zeta[1] = -17.0 / 60.0; c->zeta[2] = -5.0 / 12.0;
    c->adv_cfl_limit = sqrt(3.0);
  }
  c->time = 0.0;
  c->dt = cfg->dt0;
  so_rplan_init(&c->px, c->nx);
  so_rplan_init(&c->pxr_y, c->ny);
  so_rplan_init(&c->pzr, c->nz);
  so_cplan_init(&c->py, c->ny);
  so_cplan_init(&c->pz, c->nz);
  size_t nzb = (size_t)c->ny_min * c->nx_min * c->nze * c->lu;
  size_t nuu = (size_t)c->nx * c->ny * c->nz * c->lr;
  c->zb = (so_cplx *)calloc(nzb, sizeof(so_cplx));
  c->uu = (double *)calloc(nuu, sizeof(double));
  c->usav = (so_cplx *)calloc((size_t)c->nz_min * c->ny_min * c->nx_min * 2, sizeof(so_cplx));
  return c;
}

void so_destroy(so_ctx *c) {
  if (!c) return;
  so_rplan_free(&c->px); so_rplan_free(&c->pxr_y); so_rplan_free(&c->pzr);
  so_cplan_free(&c->py); so_cplan_free(&c->pz);
  free(c->k_x); free(c->k_y); free(c->k_z);
  free(c->zb); free(c->uu); free(c->usav);
  free(c->les_w); free(c->les_zb); free(c->les_g); free(c->les_uh); free(c->les_vt); free(c->les_cf);
  free(c);
}

void so_dims(const so_ctx *c, int *o) {
  o[0] = c->nx_min; o[1] = c->ny_min; o[2] = c->nz_min; o[3] = c->nze; o[4] = c->lu;
  o[5] = c->lr; o[6] = c->kx_max; o[7] = c->ky_max; o[8] = c->kz_max; o[9] = c->lm; o[10] = c->nx2;
}

void so_set_time(so_ctx *c, double time, double dt) { c->time = time; c->dt = dt; }

void so_stats(const so_ctx *c, double *o) {
  o[0] = c->time; o[1] = c->dt;
  for (int n = 0; n < 4; ++n) { o[2 + n] = c->u_avg[n]; o[6 + n] = c->u_var[n]; o[10 + n] = c->u_max[n]; }
  o[14] = c->energy; o[15] = c->cfl_x; o[16] = c->cfl_y; o[17] = c->cfl_z;
}

/* ------------------------------------------------------------- transforms */

/* z_trans_b.f:26-52 (isymm = 0): pad kz to Nz, cfftb, scatter into the
 * (Ny_min, nxp, Nze, n_var) block layout. */
int so_z_trans_b(so_ctx *c, const double *u1d, double *u2d, int n_var) {
  const so_cplx *u1 = (const so_cplx *)u1d;
  so_cplx *u2 = (so_cplx *)u2d;
  const int ke1 = c->kz_max + 1, ks3 = c->nze - c->nz_min;
  set_threads(c);
#pragma omp parallel
  {
    so_cplx *uc = (so_cplx *)malloc(sizeof(so_cplx) * (size_t)c->nze * 2);
    so_cplx *wk = uc + c->nze;
#pragma omp for collapse(2) schedule(static)
    for (int n = 0; n < n_var; ++n)
      for (int i = 0; i < c->nx_min; ++i)
        for (int j = 0; j < c->ny_min; ++j) {
          for (int k = 0; k < ke1; ++k) uc[k] = u1[W_IDX(c, k, j, i, n)];
          for (int k = ke1; k < ke1 + ks3; ++k) uc[k] = 0;
          for (int k = ke1 + ks3; k < c->nz; ++k) uc[k] = u1[W_IDX(c, k - ks3, j, i, n)];
          so_cfftb(&c->pz, uc, wk);
          for (int k = 0; k < c->nze; ++k) u2[ZB_IDX(c, j, i, k, n)] = uc[k];
        }
    free(uc);
  }
  return 0;
}

/* x2z_decomp.f:59-152 with one rank: the all-to-all is a self copy, then the
 * (Ny_min, Nx_min, nzp, n_var) blocks are reordered into (Ny, Nx/2, nzp, n_var)
 * with zeros for the truncated ky band.  Columns kx >= Nx_min are left as they
 * were, as in the reference. */
int so_x2z_decomp(so_ctx *c, const double *u1d, double *u2d, int n_var) {
  const so_cplx *u1 = (const so_cplx *)u1d;
  so_cplx *u2 = (so_cplx *)u2d;
  const int js3 = c->ny - c->ny_min, je1 = c->ky_max + 1;
  /* u2 may alias u1's storage only in the reference's padded arrays; the
   * restatement reads from a copy to keep aliasing harmless. */
  size_t nin = (size_t)c->ny_min * c->nx_min * c->nze * n_var;
  so_cplx *u3 = (so_cplx *)malloc(sizeof(so_cplx) * nin);
  memcpy(u3, u1, sizeof(so_cplx) * nin);
  set_threads(c);
#pragma omp parallel for collapse(2) schedule(static)
  for (int n = 0; n < n_var; ++n)
    for (int k = 0; k < c->nz; ++k)
      for (int i = 0; i < c->nx_min; ++i) {
        for (int j = 0; j < je1; ++j) u2[XY_IDX(c, j, i, k, n)] = u3[ZB_IDX(c, j, i, k, n)];
        for (int j = je1; j < je1 + js3; ++j) u2[XY_IDX(c, j, i, k, n)] = 0;
        for (int j = je1 + js3; j < c->ny; ++j) u2[XY_IDX(c, j, i, k, n)] = u3[ZB_IDX(c, j - js3, i, k, n)];
      }
  free(u3);
  return 0;
}

/* xy_trans_b.f:11-63: per (z, var) plane, cfftb along y for kx <= kx_max
 * (in place in u1), pack into the rfft layout (real part only for kx = 0),
 * zero kx > kx_max, rfftb along x.  u1 and u2 may be the same array. */
int so_xy_trans_b(so_ctx *c, double *u1d, double *u2, int n_var) {
  so_cplx *u1 = (so_cplx *)u1d;
  const int nx = c->nx, ny = c->ny, ld = nx + 1;
  set_threads(c);
#pragma omp parallel
  {
    double *work = (double *)malloc(sizeof(double) * (size_t)ld * ny);
    so_cplx *fw = (so_cplx *)malloc(sizeof(so_cplx) * (size_t)(2 * (nx > ny ? nx : ny) + 4));
#pragma omp for collapse(2) schedule(static)
    for (int n = 0; n < n_var; ++n)
      for (int k = 0; k < c->nz; ++k) {
        so_cplx *pc = u1 + XY_IDX(c, 0, 0, k, n);
        for (int i = 0; i <= c->kx_max; ++i) {
          so_cfftb(&c->py, pc + (size_t)ny * i, fw);
          for (int j = 0; j < ny; ++j) {
            so_cplx v = pc[(size_t)ny * i + j];
            if (i == 0) {
              work[(size_t)ld * j] = creal(v);
            } else {
              work[2 * i - 1 + (size_t)ld * j] = creal(v);
              work[2 * i + (size_t)ld * j] = cimag(v);
            }
          }
        }
        for (int j = 0; j < ny; ++j)
          for (int i = 2 * c->kx_max + 1; i < nx; ++i) work[i + (size_t)ld * j] = 0.0;
        double *pr = u2 + P_IDX(c, 0, 0, k, n);
        for (int j = 0; j < ny; ++j) {
          so_rfftb(&c->px, work + (size_t)ld * j, fw);
          memcpy(pr + (size_t)nx * j, work + (size_t)ld * j, sizeof(double) * nx);
        }
      }
    free(work); free(fw);
  }
  return 0;
}

/* xy_trans_f.f:13-57: per (z, var) plane, rfftf along x (in place in u1),
 * keep kx <= kx_max scaled by 1/(Nx Ny), cfftf along y, keep |ky| <= ky_max,
 * store as (nzp, Ny_min, Nx_min, n_var). */
int so_xy_trans_f(so_ctx *c, double *u1, double *u2d, int n_var) {
  so_cplx *u2 = (so_cplx *)u2d;
  const int nx = c->nx, ny = c->ny;
  const int js2 = ny - c->ny_min, je1 = c->ky_max + 1;
  const double fn = 1.0 / ((double)nx * (double)ny);
  const int ilim = c->kx_max < c->nx2 - 1 ? c->kx_max : c->nx2 - 1;
  set_threads(c);
#pragma omp parallel
  {
    so_cplx *work = (so_cplx *)malloc(sizeof(so_cplx) * (size_t)ny * (c->nx2 + 1));
    so_cplx *fw = (so_cplx *)malloc(sizeof(so_cplx) * (size_t)(2 * (nx > ny ? nx : ny) + 4));
#pragma omp for collapse(2) schedule(static)
    for (int n = 0; n < n_var; ++n)
      for (int k = 0; k < c->nz; ++k) {
        double *pr = u1 + P_IDX(c, 0, 0, k, n);
        for (int j = 0; j < ny; ++j) {
          double *line = pr + (size_t)nx * j;
          so_rfftf(&c->px, line, fw);
          work[j] = line[0] * fn;
          for (int i = 1; i <= ilim; ++i) work[j + (size_t)ny * i] = (line[2 * i - 1] + line[2 * i] * I) * fn;
          if (c->kx_max == c->nx2) work[j + (size_t)ny * c->nx2] = line[nx - 1] * fn;
        }
        for (int i = 0; i < c->nx_min; ++i) {
          so_cplx *col = work + (size_t)ny * i;
          so_cfftf(&c->py, col, fw);
          for (int j = 0; j < je1; ++j) u2[W_IDX(c, k, j, i, n)] = col[j];
          for (int j = je1; j < c->ny_min; ++j) u2[W_IDX(c, k, j, i, n)] = col[j + js2];
        }
      }
    free(work); free(fw);
  }
  return 0;
}

/* z2x_decomp.f:38-68 with one rank: the blocks (nzp, Ny_min, nxp, n_var) are
 * already (Nze, Ny_min, nxp, n_var), so the transpose is a copy. */
int so_z2x_decomp(so_ctx *c, const double *u1, double *u2, int n_var) {
  size_t n = (size_t)c->nze * c->ny_min * c->nx_min * n_var * 2;
  if (u1 != u2) memmove(u2, u1, sizeof(double) * n);
  return 0;
}

/* z_trans_f.f:21-31 (isymm = 0): cfftf along z, keep |kz| <= kz_max scaled
 * by 1/Nz in the first Nz_min rows. */
int so_z_trans_f(so_ctx *c, double *ud, int n_var) {
  so_cplx *u = (so_cplx *)ud;
  const int ke1 = c->kz_max + 1, ks2 = c->nze - c->nz_min;
  const double nz_inv = 1.0 / (double)c->nz;
  set_threads(c);
#pragma omp parallel
  {
    so_cplx *fw = (so_cplx *)malloc(sizeof(so_cplx) * (size_t)c->nze);
#pragma omp for collapse(2) schedule(static)
    for (int n = 0; n < n_var; ++n)
      for (int i = 0; i < c->nx_min; ++i)
        for (int j = 0; j < c->ny_min; ++j) {
          so_cplx *line = u + W_IDX(c, 0, j, i, n);
          so_cfftf(&c->pz, line, fw);
          for (int k = 0; k < ke1; ++k) line[k] = line[k] * nz_inv;
          for (int k = ke1; k < c->nz_min; ++k) line[k] = line[k + ks2] * nz_inv;
        }
    free(fw);
  }
  return 0;
}

/* ---------------------------------------------------------------- physics */

/* vel_max.f:11-49: FP64 sum, sum of squares and max |u| per field, then
 * averages, variances, energy, CFL numbers and (i_cfl = 1) the new dt. */
int so_vel_max(so_ctx *c, const double *u) {
  const size_t np = (size_t)c->nx * c->ny * c->nz;
  for (int n = 0; n < c->lu; ++n) {
    double s1 = 0, s2 = 0, mx = 0;
    const double *f = u + np * n;
    set_threads(c);
#pragma omp parallel for reduction(+ : s1, s2) reduction(max : mx) schedule(static)
    for (size_t p = 0; p < np; ++p) {
      double v = f[p];
      s1 += v;
      s2 += v * v;
      double a = fabs(v);
      if (a > mx) mx = a;
    }
    double inv = 1.0 / ((double)c->nx * c->ny * c->nz);
    c->u_avg[n] = s1 * inv;
    c->u_var[n] = s2 * inv - c->u_avg[n] * c->u_avg[n];
    c->u_max[n] = mx;
  }
  c->energy = 0.5 * (c->u_var[0] + c->u_var[1] + c->u_var[2]);
  double cx = c->u_max[0] * c->kx_max * c->wave_x;
  double cy = c->u_max[1] * c->ky_max * c->wave_y;
  double cz = c->u_max[2] * c->kz_max * c->wave_z;
  if (c->cfg.i_cfl == 1) {
    double cb = cx > cy ? cx : cy;
    if (cz > cb) cb = cz;
    c->dt = c->cfg.cfl0 * c->adv_cfl_limit / cb;
  }
  c->cfl_x = cx * c->dt; c->cfl_y = cy * c->dt; c->cfl_z = cz * c->dt;
  return 0;
}

static void so_les_fields(so_ctx *c, const so_cplx *u);
static double delta_sq_of(const so_ctx *c);
static void periodicity3(const so_ctx *c, double *f);
static void so_les_stress(so_ctx *c, const double *uu, int nrk);

/* rhs.f:11-142.  On entry uu(Nx,Ny,Nz,Lr) holds the physical fields in its
 * first Lu slots.  On exit r(:,:,:,1..Lu) holds the projected right-hand side
 * and r(:,:,:,Lu+1) the pressure. */
int so_rhs(so_ctx *c, double *uu, double *rd, const double *usd, int nrk) {
  so_cplx *r = (so_cplx *)rd;
  const so_cplx *usav = (const so_cplx *)usd;
  if (nrk == 1) so_vel_max(c, uu);
  const size_t np = (size_t)c->nx * c->ny * c->nz;
  const int les = c->les_stage;
  if (les) so_les_stress(c, uu, nrk);
  const double *g = c->les_g;
  /* rhs.f:32-61: the nine (six) products in upper-triangle column order */
  set_threads(c);
#pragma omp parallel for schedule(static)
  for (size_t p = 0; p < np; ++p) {
    double a = uu[p], b = uu[p + np], d = uu[p + 2 * np];
    if (c->cfg.i_strat) {
      double t = uu[p + 3 * np];
      uu[p + 8 * np] = d * t;
      uu[p + 7 * np] = b * t;
      uu[p + 6 * np] = a * t;
    }
    uu[p + 5 * np] = d * d;
    uu[p + 4 * np] = b * d;
    uu[p + 3 * np] = a * d;
    uu[p + 2 * np] = b * b;
    uu[p + 1 * np] = a * b;
    uu[p] = a * a;
    if (les)
      for (int m = 0; m < c->lr; ++m) uu[p + m * np] += g[p + m * np];
  }
  so_xy_trans_f(c, uu, rd, c->lr);
  so_z2x_decomp(c, rd, rd, c->lr);
  so_z_trans_f(c, rd, c->lr);
  /* rhs.f:74-142: stress divergence, buoyancy, projection */
  const int lu = c->lu;
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i < c->nx_min; ++i)
    for (int j = 0; j < c->ny_min; ++j) {
      double rkx = c->wave_x * c->k_x[i];
      double rkx2 = rkx * rkx;
      double rky = c->wave_y * c->k_y[j];
      double rk_sq2 = rkx2 + rky * rky;
      for (int k = 0; k < c->nz_min; ++k) {
        double rkz = c->wave_z * c->k_z[k];
        double rk_sq = rk_sq2 + rkz * rkz;
        if (rk_sq < 1.0e-10) rk_sq = 1.0e-10;
        so_cplx t[9];
        for (int n = 0; n < c->lr; ++n) t[n] = r[W_IDX(c, k, j, i, n)];
        so_cplx r1 = -I * (rkx * t[0] + rky * t[1] + rkz * t[3]);
        so_cplx r2 = -I * (rkx * t[1] + rky * t[2] + rkz * t[4]);
        so_cplx r3 = -I * (rkx * t[3] + rky * t[4] + rkz * t[5]);
        if (c->cfg.i_strat) {
          size_t is = (size_t)k + (size_t)c->nz_min * ((size_t)j + (size_t)c->ny_min * (size_t)i);
          size_t st = (size_t)c->nz_min * c->ny_min * c->nx_min;
          so_cplx wsav = usav[is], tsav = usav[is + st];
          r1 += c->cfg.buoy_fac_x * tsav;
          r3 += c->cfg.buoy_fac_z * tsav;
          so_cplx r4 = -I * (rkx * t[6] + rky * t[7] + rkz * t[8]) - c->cfg.lapse * wsav;
          r[W_IDX(c, k, j, i, 3)] = r4;
        }
        so_cplx p = -I * (rkx * r1 + rky * r2 + rkz * r3) / rk_sq;
        r[W_IDX(c, k, j, i, 0)] = r1 - I * rkx * p;
        r[W_IDX(c, k, j, i, 1)] = r2 - I * rky * p;
        r[W_IDX(c, k, j, i, 2)] = r3 - I * rkz * p;
        r[W_IDX(c, k, j, i, lu)] = p;
      }
    }
  return 0;
}

/* sam.f:169-314 without the output branches: transform u to physical space,
 * save (w, T), pre-update with the previous rhs, rhs, RK update with the
 * viscous integrating factor.  r must hold Lr fields (Nze,Ny_min,Nx_min). */
int so_stage(so_ctx *c, double *ud, double *rd, int nrk) {
  so_cplx *u = (so_cplx *)ud;
  so_cplx *r = (so_cplx *)rd;
  const int lu = c->lu;
  so_z_trans_b(c, ud, (double *)c->zb, lu);
  if (c->les_model) {
    /* gradient fields of the current u to physical space */
    const int ng = c->lr + (c->les_model == 3 ? 3 : 0);
    so_les_fields(c, u);
    so_z_trans_b(c, (const double *)c->les_w, (double *)c->les_zb, ng);
    so_x2z_decomp(c, (const double *)c->les_zb, c->les_g, ng);
    so_xy_trans_b(c, c->les_g, c->les_g, ng);
    c->les_stage = 1;
  }
  if (c->cfg.i_strat) {
    /* sam.f:175-195 */
    size_t st = (size_t)c->nz_min * c->ny_min * c->nx_min;
    for (int i = 0; i < c->nx_min; ++i)
      for (int j = 0; j < c->ny_min; ++j)
        for (int k = 0; k < c->nz_min; ++k) {
          size_t is = (size_t)k + (size_t)c->nz_min * ((size_t)j + (size_t)c->ny_min * (size_t)i);
          so_cplx w = u[W_IDX(c, k, j, i, 2)];
          if (c->cfg.rot_sav) w = c->cfg.cos_theta * w - c->cfg.sin_theta * u[W_IDX(c, k, j, i, 0)];
          c->usav[is] = w;
          c->usav[is + st] = u[W_IDX(c, k, j, i, 3)];
        }
  }
  /* sam.f:210-221 */
  const double dt_fac2 = c->zeta[nrk - 1] * c->dt;
  if (nrk > 1) {
    for (int n = 0; n < lu; ++n)
      for (int i = 0; i < c->nx_min; ++i)
        for (int j = 0; j < c->ny_min; ++j)
          for (int k = 0; k < c->nz_min; ++k) u[W_IDX(c, k, j, i, n)] += dt_fac2 * r[W_IDX(c, k, j, i, n)];
  }
  /* sam.f:226-232 */
  so_x2z_decomp(c, (const double *)c->zb, c->uu, lu);
  so_xy_trans_b(c, c->uu, c->uu, lu);
  /* sam.f:244 */
  so_rhs(c, c->uu, rd, (const double *)c->usav, nrk);
  c->les_stage = 0;
  /* sam.f:293-314 */
  const double dt_fac1 = c->gamma[nrk - 1] * c->dt;
  const double dt_fac = dt_fac1 + dt_fac2;
  double vis_f = c->cfg.vis * dt_fac;
  for (int n = 0; n < lu; ++n) {
    if (n == 3) vis_f = vis_f * c->pr_inv;
    set_threads(c);
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 0; i < c->nx_min; ++i)
      for (int j = 0; j < c->ny_min; ++j) {
        double rkx = c->wave_x * c->k_x[i];
        double rkx2 = rkx * rkx;
        double rky = c->wave_y * c->k_y[j];
        double rk_sq2 = rkx2 + rky * rky;
        for (int k = 0; k < c->nz_min; ++k) {
          double rkz = c->wave_z * c->k_z[k];
          double rk_sq = rk_sq2 + rkz * rkz;
          double vis_fac = exp(-vis_f * rk_sq);
          size_t id = W_IDX(c, k, j, i, n);
          u[id] = (u[id] + dt_fac1 * r[id]) * vis_fac;
        }
      }
  }
  return 0;
}

static void so_ou_apply(so_ctx *c, double *ud);

int so_steps(so_ctx *c, double *u, double *r, int nsteps) {
  for (int s = 0; s < nsteps; ++s) {
    for (int nrk = 1; nrk <= c->cfg.nrk_max; ++nrk) so_stage(c, u, r, nrk);
    c->time += c->dt; /* sam.f:318 */
    if (c->ou_n > 0) so_ou_apply(c, u);
  }
  return 0;
}

/* ------------------------------------------------------------ diagnostics */

/* spectra.f:13-90: shell sums of E(k), T(k), D(k), Chollet-Lesieur nu_t(k),
 * mode count, and divergence rms / max. */
int so_spectra(so_ctx *c, const double *ud, const double *rd, double *out) {
  const so_cplx *u = (const so_cplx *)ud, *r = (const so_cplx *)rd;
  const int lm = c->lm;
  double *w = (double *)calloc((size_t)lm * 5, sizeof(double));
  double div_sum = 0.0, div_mx = 0.0;
  double fac_cl = 0.0;
  if (c->cfg.i_les) fac_cl = sqrt(2.0 * so_cl_energy(c, ud) / (double)c->k_cl);
  for (int n = 0; n < c->lu; ++n) c->u_avg[n] = creal(u[W_IDX(c, 0, 0, 0, n)]);
  for (int i = 0; i < c->nx_min; ++i) {
    double factor = (i == 0 || i == c->nx2) ? 1.0 : 2.0;
    int kx2 = c->k_x[i] * c->k_x[i];
    double rkx = c->wave_x * c->k_x[i];
    double rkx2 = rkx * rkx;
    for (int j = 0; j < c->ny_min; ++j) {
      int k_sq2 = kx2 + c->k_y[j] * c->k_y[j];
      double rky = c->wave_y * c->k_y[j];
      double rk_sq2 = rkx2 + rky * rky;
      for (int k = 0; k < c->nz_min; ++k) {
        int k_sq = k_sq2 + c->k_z[k] * c->k_z[k];
        double k_mag = sqrt((double)k_sq);
        int is = (int)(k_mag + 0.5);
        double rkz = c->wave_z * c->k_z[k];
        double rk_sq = rk_sq2 + rkz * rkz;
        double vist = 0.0;
        if (!(k_sq == 0 || c->cfg.i_les == 0))
          vist = fac_cl * (c->a_cl + c->b_cl * exp(-(c->c_cl * c->k_cl) / k_mag));
        so_cplx u1 = u[W_IDX(c, k, j, i, 0)], u2 = u[W_IDX(c, k, j, i, 1)], u3 = u[W_IDX(c, k, j, i, 2)];
        double u_sq = creal(u1 * conj(u1) + u2 * conj(u2) + u3 * conj(u3));
        double udu = creal(r[W_IDX(c, k, j, i, 0)] * conj(u1) + r[W_IDX(c, k, j, i, 1)] * conj(u2) +
                           r[W_IDX(c, k, j, i, 2)] * conj(u3));
        w[is + lm * 0] += factor * u_sq;
        w[is + lm * 1] += factor * udu;
        w[is + lm * 2] += factor * rk_sq * (c->cfg.vis + vist) * u_sq;
        w[is + lm * 3] += factor * vist;
        w[is + lm * 4] += factor;
        so_cplx div = rkx * u1 + rky * u2 + rkz * u3;
        double div_sq = creal(div * conj(div));
        div_sum += div_sq;
        if (div_sq > div_mx) div_mx = div_sq;
      }
    }
  }
  double sum_ek = 0.0;
  for (int s = 0; s < lm; ++s) sum_ek += w[s];
  memcpy(out, w, sizeof(double) * (size_t)lm * 5);
  out[5 * lm + 0] = 0.5 * sum_ek;
  out[5 * lm + 1] = sqrt(div_sum);
  out[5 * lm + 2] = sqrt(div_mx);
  free(w);
  return 0;
}

/* div_check.f:11-36 */
int so_div_check(so_ctx *c, const double *ud, double *o) {
  const so_cplx *u = (const so_cplx *)ud;
  double s[4] = {0, 0, 0, 0};
  for (int i = 0; i < c->nx_min; ++i) {
    double rkx = c->wave_x * c->k_x[i];
    for (int j = 0; j < c->ny_min; ++j) {
      double rky = c->wave_y * c->k_y[j];
      for (int k = 0; k < c->nz_min; ++k) {
        double rkz = c->wave_z * c->k_z[k];
        so_cplx div = rkx * u[W_IDX(c, k, j, i, 0)] + rky * u[W_IDX(c, k, j, i, 1)] + rkz * u[W_IDX(c, k, j, i, 2)];
        double div_sq = creal(div * conj(div));
        s[0] += sqrt(div_sq);
        s[1] += div_sq;
        if (div_sq > s[2]) s[2] = div_sq;
        if (div_sq > 1.e-20) s[3] += 1.0;
      }
    }
  }
  o[0] = s[0]; o[1] = sqrt(s[1]); o[2] = sqrt(s[2]); o[3] = s[3];
  return 0;
}

/* cl_energy.f:8-43.  Rows beyond Nz_min of the padded z dimension are the
 * reference's padding; they are read as stored (zero after read_field). */
double so_cl_energy(so_ctx *c, const double *ud) {
  const so_cplx *u = (const so_cplx *)ud;
  double cl_start_sq = ((double)c->k_cl - 0.5) * ((double)c->k_cl - 0.5);
  double cl_stop_sq = ((double)c->k_cl + 0.5) * ((double)c->k_cl + 0.5);
  double sum_e = 0.0;
  for (int i = 0; i < c->nx_min; ++i) {
    double factor = (i == 0 || i == c->nx / 2) ? 1.0 : 2.0;
    int kx2 = c->k_x[i] * c->k_x[i];
    for (int j = 0; j < c->ny_min; ++j) {
      int k_sq2 = kx2 + c->k_y[j] * c->k_y[j];
      int k_start = k_sq2 > cl_start_sq ? 1 : (int)sqrt(cl_start_sq - k_sq2) + 2;
      int k_stop = k_sq2 > cl_stop_sq ? 0 : (int)sqrt(cl_stop_sq - k_sq2) + 1;
      for (int k1 = k_start; k1 <= k_stop; ++k1) { /* 1-based as in the reference */
        int kk1 = c->nz_min + 2 - k1;
        int k = k1 - 1, kk = kk1 - 1;
        double s1 = 0.0, s2 = 0.0;
        for (int n = 0; n < 3; ++n) {
          so_cplx a = (k < c->nze) ? u[W_IDX(c, k, j, i, n)] : 0;
          so_cplx b = (kk < c->nze && kk >= 0) ? u[W_IDX(c, kk, j, i, n)] : 0;
          s1 += creal(a * conj(a));
          s2 += creal(b * conj(b));
        }
        sum_e += factor * (s1 + s2);
      }
    }
  }
  return sum_e;
}

/* get_mean.f:8-56 (i_symm = 0): horizontal-mean profile through rfftb in z
 * and the linear-jump estimate; i_remove = 1 subtracts the jump's linear
 * profile from the kx = ky = 0 column. */
double so_get_mean(so_ctx *c, double *ud, int i_remove, double *u_mean) {
  so_cplx *u = (so_cplx *)ud; /* one field (Nze, Ny_min, Nx_min) */
  const int nz = c->nz;
  const double nz_inv = 1.0 / nz;
  so_cplx *fw = (so_cplx *)malloc(sizeof(so_cplx) * (size_t)(2 * nz + 4));
  double *work = (double *)malloc(sizeof(double) * (size_t)nz);
  double jump = 0.0;
  for (int pass = 0; pass < 2; ++pass) {
    u_mean[0] = creal(u[0]);
    for (int k = 1; k <= c->kz_max; ++k) { u_mean[2 * k - 1] = creal(u[k]); u_mean[2 * k] = cimag(u[k]); }
    for (int k = 2 * c->kz_max + 1; k < nz; ++k) u_mean[k] = 0.0;
    so_rfftb(&c->pzr, u_mean, fw);
    double u_n = 3.0 * u_mean[0] - 3.0 * u_mean[1] + u_mean[2];
    double u_1 = 3.0 * u_mean[nz - 1] - 3.0 * u_mean[nz - 2] + u_mean[nz - 3];
    double jmp = 0.5 * ((u_mean[nz - 1] - u_n) + (u_1 - u_mean[0]));
    if (pass == 0) {
      jump = jmp;
      if (i_remove != 1) break;
      for (int k = 0; k < nz; ++k) work[k] = jump * ((double)k * nz_inv - 0.5);
      so_rfftf(&c->pzr, work, fw);
      for (int k = 0; k <= c->kz_max; ++k) work[k] = work[k] * nz_inv;
      u[0] -= work[0];
      for (int k = 1; k <= c->kz_max; ++k) {
        int k2 = c->nz_min - k;
        u[k] -= work[2 * k - 1] + work[2 * k] * I;
        u[k2] -= work[2 * k - 1] - work[2 * k] * I;
      }
    } else {
      jump = jump - jmp;
    }
  }
  free(fw); free(work);
  return jump;
}

/* ------------------------------------------------------ plane derivatives */

/* x_deriv.f:7-25 */
int so_x_deriv(so_ctx *c, const double *u, double *du) {
  const int nx = c->nx, ny = c->ny;
  so_cplx *fw = (so_cplx *)malloc(sizeof(so_cplx) * (size_t)(2 * nx + 4));
  const double nx_inv = 1.0 / nx;
  for (int j = 0; j < ny; ++j) {
    double *d = du + (size_t)nx * j;
    for (int i = 0; i < nx; ++i) d[i] = u[(size_t)nx * j + i] * nx_inv;
    so_rfftf(&c->px, d, fw);
    d[0] = 0.0;
    for (int i = 1; i <= c->kx_max; ++i) {
      double rkx = c->k_x[i] * c->wave_x;
      double tmp = d[2 * i - 1];
      d[2 * i - 1] = -rkx * d[2 * i];
      d[2 * i] = rkx * tmp;
    }
    for (int i = 2 * c->kx_max + 1; i < nx; ++i) d[i] = 0.0;
    so_rfftb(&c->px, d, fw);
  }
  free(fw);
  return 0;
}

/* y_deriv.f:7-28 */
int so_y_deriv(so_ctx *c, const double *u, double *du) {
  const int nx = c->nx, ny = c->ny;
  so_cplx *fw = (so_cplx *)malloc(sizeof(so_cplx) * (size_t)(2 * ny + 4));
  double *work = (double *)malloc(sizeof(double) * (size_t)ny);
  const double ny_inv = 1.0 / ny;
  for (int i = 0; i < nx; ++i) {
    for (int j = 0; j < ny; ++j) work[j] = u[(size_t)nx * j + i] * ny_inv;
    so_rfftf(&c->pxr_y, work, fw);
    work[0] = 0.0;
    for (int j = 1; j <= c->ky_max; ++j) {
      double rky = c->k_y[j] * c->wave_y;
      double tmp = work[2 * j - 1];
      work[2 * j - 1] = -rky * work[2 * j];
      work[2 * j] = rky * tmp;
    }
    for (int j = 2 * c->ky_max + 1; j < ny; ++j) work[j] = 0.0;
    so_rfftb(&c->pxr_y, work, fw);
    for (int j = 0; j < ny; ++j) du[(size_t)nx * j + i] = work[j];
  }
  free(fw); free(work);
  return 0;
}

/* --------------------------------------------- subgrid models (haloed grids)
 * filter.f, sm.f, dm.f include a header (speciso.h) that the reference does
 * not ship.  Its symbols are defined here from their use:
 *   Lx = Nx+2, Ly = Ny+2, Lz = Nz+2 (periodic halo planes 1 and N+2,
 *     periodicity.f:7-32);
 *   ifact = (1,1,1,2,2,2) for the symmetric tensor (S11,S22,S33,S12,S23,S13);
 *   ip = (1,2,3,1,2,1), jp = (1,2,3,2,3,3) the index pairs of that tensor;
 *   alpha_sq = 4 (test-to-grid filter width ratio 2 for the 1-4-1 filter);
 *   delta_sq = (dx dy dz)^(2/3) (init.f:28), dx = xL/Nx etc.;
 *   c_smag from the input deck (sam.h /static/).
 */
#define H2(c, i, j) ((size_t)(i) + (size_t)((c)->nx + 2) * (size_t)(j))
#define H3(c, i, j, k) (H2(c, i, j) + (size_t)((c)->nx + 2) * ((c)->ny + 2) * (size_t)(k))

static const int SO_IFACT[6] = {1, 1, 1, 2, 2, 2};
static const int SO_IP[6] = {0, 1, 2, 0, 1, 0};
static const int SO_JP[6] = {0, 1, 2, 1, 2, 2};
static const double SO_ALPHA_SQ = 4.0;

/* periodicity2.f:7-19 on a plane array f(Lx,Ly,n_var) */
static void periodicity2(const so_ctx *c, double *f, int n_var) {
  const int nx = c->nx, ny = c->ny;
  const size_t pl = (size_t)(nx + 2) * (ny + 2);
  for (int n = 0; n < n_var; ++n) {
    double *g = f + pl * n;
    for (int j = 1; j <= ny; ++j) { g[H2(c, nx + 1, j)] = g[H2(c, 1, j)]; g[H2(c, 0, j)] = g[H2(c, nx, j)]; }
    for (int i = 0; i < nx + 2; ++i) { g[H2(c, i, ny + 1)] = g[H2(c, i, 1)]; g[H2(c, i, 0)] = g[H2(c, i, ny)]; }
  }
}

/* periodicity.f:7-32 on a volume f(Lx,Ly,Lz) */
static void periodicity3(const so_ctx *c, double *f) {
  const int nx = c->nx, ny = c->ny, nz = c->nz;
  for (int j = 1; j <= ny; ++j)
    for (int k = 1; k <= nz; ++k) { f[H3(c, nx + 1, j, k)] = f[H3(c, 1, j, k)]; f[H3(c, 0, j, k)] = f[H3(c, nx, j, k)]; }
  for (int i = 0; i < nx + 2; ++i)
    for (int k = 1; k <= nz; ++k) { f[H3(c, i, ny + 1, k)] = f[H3(c, i, 1, k)]; f[H3(c, i, 0, k)] = f[H3(c, i, ny, k)]; }
  for (int i = 0; i < nx + 2; ++i)
    for (int j = 0; j < ny + 2; ++j) { f[H3(c, i, j, nz + 1)] = f[H3(c, i, j, 1)]; f[H3(c, i, j, 0)] = f[H3(c, i, j, nz)]; }
}

/* filter.f:7-42: 1-4-1 across the three planes of f_bar(Lx,Ly,n_var,3), then
 * along y, then along x, normalised by 1/6^3. */
int so_filter(so_ctx *c, const double *f_bar, double *f_hat, int n_var) {
  const int nx = c->nx, ny = c->ny;
  const size_t pl = (size_t)(nx + 2) * (ny + 2);
  const double w_inv = 1.0 / ((1.0 + 4.0 + 1.0) * (1.0 + 4.0 + 1.0) * (1.0 + 4.0 + 1.0));
  int lw = (nx > ny ? nx : ny) + 2;
  double *w_r = (double *)malloc(sizeof(double) * (size_t)lw);
  for (int n = 0; n < n_var; ++n)
    for (int i = 0; i < nx + 2; ++i)
      for (int j = 0; j < ny + 2; ++j)
        f_hat[H2(c, i, j) + pl * n] = f_bar[H2(c, i, j) + pl * n] + 4 * f_bar[H2(c, i, j) + pl * (n + n_var)] +
                                      f_bar[H2(c, i, j) + pl * (n + 2 * n_var)];
  for (int n = 0; n < n_var; ++n)
    for (int i = 1; i <= nx; ++i) {
      for (int j = 0; j < ny + 2; ++j) w_r[j] = f_hat[H2(c, i, j) + pl * n];
      for (int j = 1; j <= ny; ++j) f_hat[H2(c, i, j) + pl * n] = w_r[j - 1] + 4 * w_r[j] + w_r[j + 1];
    }
  periodicity2(c, f_hat, n_var);
  for (int n = 0; n < n_var; ++n)
    for (int j = 1; j <= ny; ++j) {
      for (int i = 0; i < nx + 2; ++i) w_r[i] = f_hat[H2(c, i, j) + pl * n];
      for (int i = 1; i <= nx; ++i) f_hat[H2(c, i, j) + pl * n] = w_inv * (w_r[i - 1] + 4 * w_r[i] + w_r[i + 1]);
    }
  periodicity2(c, f_hat, n_var);
  free(w_r);
  return 0;
}

/* the staggered-to-centre velocity of one haloed plane kk (sm.f:45-51) */
static void centre_plane(const so_ctx *c, const double *u, int kk, double *ub) {
  const int nx = c->nx, ny = c->ny;
  const size_t pl = (size_t)(nx + 2) * (ny + 2), vol = pl * (c->nz + 2);
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j) {
      ub[H2(c, i, j)] = 0.5 * (u[H3(c, i, j, kk)] + u[H3(c, i - 1, j, kk)]);
      ub[H2(c, i, j) + pl] = 0.5 * (u[H3(c, i, j, kk) + vol] + u[H3(c, i, j - 1, kk) + vol]);
      ub[H2(c, i, j) + 2 * pl] = 0.5 * (u[H3(c, i, j, kk) + 2 * vol] + u[H3(c, i, j, kk - 1) + 2 * vol]);
    }
  periodicity2(c, ub, 3);
}

/* strain of the centre plane from three u_bar planes lo/mid/hi (sm.f:57-75) */
static void strain_plane(const so_ctx *c, const double *lo, const double *mid, const double *hi, double *sb) {
  const int nx = c->nx, ny = c->ny;
  const size_t pl = (size_t)(nx + 2) * (ny + 2);
  const double dx_inv = c->nx / c->cfg.xl, dy_inv = c->ny / c->cfg.yl, dz_inv = c->nz / c->cfg.zl;
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j) {
#define UB(p, ii, jj, n) (p)[H2(c, ii, jj) + pl * (n)]
      sb[H2(c, i, j)] = 0.5 * (UB(mid, i + 1, j, 0) - UB(mid, i - 1, j, 0)) * dx_inv;
      sb[H2(c, i, j) + pl] = 0.5 * (UB(mid, i, j + 1, 1) - UB(mid, i, j - 1, 1)) * dy_inv;
      sb[H2(c, i, j) + 2 * pl] = 0.5 * (UB(hi, i, j, 2) - UB(lo, i, j, 2)) * dz_inv;
      sb[H2(c, i, j) + 3 * pl] = .25 * ((UB(mid, i, j + 1, 0) - UB(mid, i, j - 1, 0)) * dy_inv +
                                        (UB(mid, i + 1, j, 1) - UB(mid, i - 1, j, 1)) * dx_inv);
      sb[H2(c, i, j) + 4 * pl] = .25 * ((UB(hi, i, j, 1) - UB(lo, i, j, 1)) * dz_inv +
                                        (UB(mid, i, j + 1, 2) - UB(mid, i, j - 1, 2)) * dy_inv);
      sb[H2(c, i, j) + 5 * pl] = .25 * ((UB(mid, i + 1, j, 2) - UB(mid, i - 1, j, 2)) * dx_inv +
                                        (UB(hi, i, j, 0) - UB(lo, i, j, 0)) * dz_inv);
#undef UB
    }
}

static double delta_sq_of(const so_ctx *c) {
  double dx = c->cfg.xl / c->nx, dy = c->cfg.yl / c->ny, dz = c->cfg.zl / c->nz;
  return pow(dx * dy * dz, 2.0 / 3.0);
}

/* sm.f:41-101: conventional Smagorinsky nu_t = c_smag delta^2 |S| */
int so_sm(so_ctx *c, const double *u, double *vt) {
  const int nx = c->nx, ny = c->ny, nz = c->nz;
  const size_t pl = (size_t)(nx + 2) * (ny + 2);
  const double c_delta_sq = c->cfg.c_smag * delta_sq_of(c);
  double *ub = (double *)calloc(pl * 9, sizeof(double));
  double *sb = (double *)calloc(pl * 6, sizeof(double));
  for (int k = 0; k <= nz + 1; ++k) {
    int kk = k + 1;
    if (kk < 2) kk += nz;
    centre_plane(c, u, kk - 1, ub + 2 * 3 * pl); /* slot 3; haloed indices are 0-based here */
    if (k >= 2) {
      strain_plane(c, ub, ub + 3 * pl, ub + 6 * pl, sb);
      for (int i = 1; i <= nx; ++i)
        for (int j = 1; j <= ny; ++j) {
          double sum = 0.0;
          for (int n = 0; n < 6; ++n) sum += SO_IFACT[n] * sb[H2(c, i, j) + pl * n] * sb[H2(c, i, j) + pl * n];
          vt[H3(c, i, j, k - 1)] = c_delta_sq * sqrt(2.0 * sum);
        }
    }
    memmove(ub, ub + 3 * pl, sizeof(double) * pl * 6);
  }
  periodicity3(c, vt);
  free(ub); free(sb);
  return 0;
}

/* dm.f:43-191: dynamic Smagorinsky (Germano identity, Lilly least squares
 * over the whole volume).  Returns c_delta_sq; vt = c_delta_sq |S|. */
double so_dm(so_ctx *c, const double *u, double *vt) {
  const int nx = c->nx, ny = c->ny, nz = c->nz;
  const size_t pl = (size_t)(nx + 2) * (ny + 2);
  double *ub = (double *)calloc(pl * 12, sizeof(double));   /* u_bar(Lx,Ly,3,4) */
  double *sb = (double *)calloc(pl * 18, sizeof(double));   /* s_bar(Lx,Ly,6,3) */
  double *sms = (double *)calloc(pl * 18, sizeof(double));  /* s_mag_s(Lx,Ly,6,3) */
  double *ubub = (double *)calloc(pl * 18, sizeof(double)); /* u_bar_u_bar(Lx,Ly,6,3) */
  double *u_hat = (double *)calloc(pl * 3, sizeof(double));
  double *s_hat = (double *)calloc(pl * 6, sizeof(double));
  double *L = (double *)calloc(pl * 6, sizeof(double));
  double *M = (double *)calloc(pl * 6, sizeof(double));
  double num = 0.0, den = 0.0;
  for (int k = -3; k <= nz + 1; ++k) {
    int kk = k + 2;
    if (kk < 2) kk += nz;
    if (kk > nz + 2) kk -= nz;
    centre_plane(c, u, kk - 1, ub + 3 * 3 * pl);
    if (k >= 0) {
      strain_plane(c, ub + 3 * pl, ub + 6 * pl, ub + 9 * pl, sb + 12 * pl);
      periodicity2(c, sb + 12 * pl, 6);
      for (int i = 1; i <= nx; ++i)
        for (int j = 1; j <= ny; ++j) {
          double sum = 0.0;
          for (int n = 0; n < 6; ++n) {
            double s = sb[H2(c, i, j) + pl * (12 + n)];
            sum += SO_IFACT[n] * s * s;
          }
          double s_mag = sqrt(2.0 * sum);
          if (k >= 1) vt[H3(c, i, j, k)] = s_mag;
          for (int n = 0; n < 6; ++n) {
            sms[H2(c, i, j) + pl * (12 + n)] = s_mag * sb[H2(c, i, j) + pl * (12 + n)];
            ubub[H2(c, i, j) + pl * (12 + n)] =
                ub[H2(c, i, j) + pl * (6 + SO_IP[n])] * ub[H2(c, i, j) + pl * (6 + SO_JP[n])];
          }
        }
      periodicity2(c, sms + 12 * pl, 6);
      periodicity2(c, ubub + 12 * pl, 6);
    }
    if (k >= 2) {
      so_filter(c, ub, u_hat, 3);
      so_filter(c, sb, s_hat, 6);
      so_filter(c, sms, M, 6);
      so_filter(c, ubub, L, 6);
      for (int i = 1; i <= nx; ++i)
        for (int j = 1; j <= ny; ++j) {
          double sum = 0.0;
          for (int n = 0; n < 6; ++n) sum += SO_IFACT[n] * s_hat[H2(c, i, j) + pl * n] * s_hat[H2(c, i, j) + pl * n];
          double s_mag = sqrt(2.0 * sum);
          for (int n = 0; n < 6; ++n) {
            size_t id = H2(c, i, j) + pl * n;
            M[id] = -M[id] + SO_ALPHA_SQ * s_mag * s_hat[id];
            L[id] = L[id] - u_hat[H2(c, i, j) + pl * SO_IP[n]] * u_hat[H2(c, i, j) + pl * SO_JP[n]];
          }
        }
      for (int i = 1; i <= nx; ++i)
        for (int j = 1; j <= ny; ++j)
          for (int n = 0; n < 6; ++n) {
            size_t id = H2(c, i, j) + pl * n;
            num += SO_IFACT[n] * L[id] * M[id];
            den += SO_IFACT[n] * M[id] * M[id];
          }
    }
    /* shift the plane slots (dm.f:154-170) */
    memmove(ub, ub + 3 * pl, sizeof(double) * pl * 9);
    memmove(sb, sb + 6 * pl, sizeof(double) * pl * 12);
    memmove(sms, sms + 6 * pl, sizeof(double) * pl * 12);
    memmove(ubub, ubub + 6 * pl, sizeof(double) * pl * 12);
  }
  double c_delta_sq = -0.5 * num / den;
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j)
      for (int k = 1; k <= nz; ++k) vt[H3(c, i, j, k)] = c_delta_sq * vt[H3(c, i, j, k)];
  periodicity3(c, vt);
  free(ub); free(sb); free(sms); free(ubub); free(u_hat); free(s_hat); free(L); free(M);
  return c_delta_sq;
}

/* ----------------------------------------------------------- initial fields */

/* splitmix64 (Steele, Lea & Flood 2014): a counter-based generator so the
 * CUDA initialiser and this oracle draw identical phases per mode. */
static uint64_t so_mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

static double so_uniform(uint64_t seed, int stream, int i, int j, int k) {
  uint64_t ctr = ((((uint64_t)stream * 4096u + (uint64_t)i) * 4096u + (uint64_t)j) * 4096u) + (uint64_t)k;
  uint64_t x = so_mix64(seed ^ so_mix64(ctr));
  return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

/* e_k (initial_field.f:324-372): kind 0 = k^2 (white), 6 = k^4 exp(-2 (k/4)^2) */
static double so_ek(double k, int kind) {
  if (kind == 6) return k * k * k * k * exp(-2.0 * (k / 4.0) * (k / 4.0));
  return k * k;
}

/* enforce_symm (initial_field.f:422-460) on the kx = 0 plane */
static void enforce_symm(so_ctx *c, so_cplx *u, int n0, int n_var) {
  for (int n = n0; n < n0 + n_var; ++n) {
    so_cplx v = u[W_IDX(c, 0, 0, 0, n)];
    u[W_IDX(c, 0, 0, 0, n)] = 0.5 * (v + conj(v));
    for (int j = c->ky_max + 1; j < c->ny_min; ++j) u[W_IDX(c, 0, j, 0, n)] = conj(u[W_IDX(c, 0, c->ny_min - j, 0, n)]);
    for (int k = c->kz_max + 1; k < c->nz_min; ++k) u[W_IDX(c, k, 0, 0, n)] = conj(u[W_IDX(c, c->nz_min - k, 0, 0, n)]);
    for (int j = 1; j < c->ny_min; ++j)
      for (int k = c->kz_max + 1; k < c->nz_min; ++k)
        u[W_IDX(c, k, j, 0, n)] = conj(u[W_IDX(c, c->nz_min - k, c->ny_min - j, 0, n)]);
  }
}

/* rescale (initial_field.f:470-494) */
static void rescale(so_ctx *c, so_cplx *u, int n0, int n_var, double flct) {
  double sum1 = 0.0;
  for (int n = n0; n < n0 + n_var; ++n)
    for (int i = 0; i < c->nx_min; ++i)
      for (int j = 0; j < c->ny_min; ++j)
        for (int k = 0; k < c->nz_min; ++k) {
          so_cplx v = u[W_IDX(c, k, j, i, n)];
          sum1 += creal(v * conj(v));
        }
  if (sum1 <= 0.0) return;
  double scale = flct * sqrt((double)n_var) / sqrt(sum1);
  for (int n = n0; n < n0 + n_var; ++n)
    for (int i = 0; i < c->nx_min; ++i)
      for (int j = 0; j < c->ny_min; ++j)
        for (int k = 0; k < c->nz_min; ++k) u[W_IDX(c, k, j, i, n)] *= scale;
}

static void zero_field(so_ctx *c, so_cplx *u) {
  memset(u, 0, sizeof(so_cplx) * (size_t)c->nze * c->ny_min * c->nx_min * c->lu);
}

/* Taylor-Green u = sin x cos y cos z, v = -cos x sin y cos z, w = 0 set
 * directly in wave space: coefficients at kx = 1, ky = +-1, kz = +-1 are
 * -i/8 for u and i sign(ky)/8 for v (exact in binary). */
int so_init_taylor_green(so_ctx *c, double *ud) {
  so_cplx *u = (so_cplx *)ud;
  zero_field(c, u);
  if (c->kx_max < 1 || c->ky_max < 1 || c->kz_max < 1) return -1;
  for (int sj = -1; sj <= 1; sj += 2)
    for (int sk = -1; sk <= 1; sk += 2) {
      int j = sj > 0 ? 1 : c->ny_min - 1;
      int k = sk > 0 ? 1 : c->nz_min - 1;
      u[W_IDX(c, k, j, 1, 0)] = -0.125 * I;
      u[W_IDX(c, k, j, 1, 1)] = 0.125 * sj * I;
    }
  return 0;
}

/* initial_field.f:62-122 velocity construction and :168-185 temperature,
 * with this build's RNG and spectra. */
int so_init_random(so_ctx *c, double *ud, unsigned long long seed, int kind_u, double flct_u, int kind_t,
                   double flct_t) {
  so_cplx *u = (so_cplx *)ud;
  zero_field(c, u);
  const double two_pi = 2.0 * SO_PI, factor = 1.0 / two_pi;
  for (int i = 0; i < c->nx_min; ++i) {
    int kx2 = c->k_x[i] * c->k_x[i];
    double rkx = c->wave_x * c->k_x[i];
    double rkx2 = rkx * rkx;
    for (int j = 0; j < c->ny_min; ++j) {
      int k_sq2 = kx2 + c->k_y[j] * c->k_y[j];
      double rky = c->wave_y * c->k_y[j];
      double rk_sq2 = rkx2 + rky * rky;
      double rk12_mag = sqrt(rk_sq2);
      for (int k = 0; k < c->nz_min; ++k) {
        int k_sq = k_sq2 + c->k_z[k] * c->k_z[k];
        double k_mag = sqrt((double)k_sq);
        double k_mag1 = k_mag > 1.0e-8 ? k_mag : 1.0e-8;
        double rkz = c->wave_z * c->k_z[k];
        double rk_sq = rk_sq2 + rkz * rkz;
        double rk_mag = sqrt(rk_sq);
        double f = sqrt(so_ek(k_mag, kind_u) * factor) / k_mag1;
        double th1 = two_pi * so_uniform(seed, 0, i, j, k);
        double th2 = two_pi * so_uniform(seed, 1, i, j, k);
        double phi = two_pi * so_uniform(seed, 2, i, j, k);
        so_cplx alpha = f * (cos(th1) + I * sin(th1)) * cos(phi);
        so_cplx beta1 = f * (cos(th2) + I * sin(th2)) * sin(phi);
        if (rk12_mag == 0.0) {
          u[W_IDX(c, k, j, i, 0)] = alpha;
          u[W_IDX(c, k, j, i, 1)] = beta1;
          u[W_IDX(c, k, j, i, 2)] = 0.0;
        } else {
          double denom = 1.0 / (rk_mag * rk12_mag);
          u[W_IDX(c, k, j, i, 0)] = (alpha * rk_mag * rky + beta1 * rkx * rkz) * denom;
          u[W_IDX(c, k, j, i, 1)] = (beta1 * rky * rkz - alpha * rk_mag * rkx) * denom;
          u[W_IDX(c, k, j, i, 2)] = -beta1 * rk12_mag / rk_mag;
        }
        if (c->lu == 4) {
          double ft = sqrt(so_ek(k_mag, kind_t) * factor) / k_mag1;
          double th = two_pi * so_uniform(seed, 3, i, j, k);
          u[W_IDX(c, k, j, i, 3)] = ft * (cos(th) + I * sin(th));
        }
      }
    }
  }
  enforce_symm(c, u, 0, 3);
  rescale(c, u, 0, 3, flct_u);
  if (c->lu == 4) {
    enforce_symm(c, u, 3, 1);
    rescale(c, u, 3, 1, flct_t);
  }
  return 0;
}

/* initial_field.f:225-248: one plane wave in the non-tilted box (i_prob=-4),
 * with zero background fluctuations and mean wind uo. */
int so_init_gw_plane(so_ctx *c, double *ud, double amplitude, double lambda_x, double lambda_z, double omega_i,
                     double k_w, double m_w, double lapse0, double uo) {
  so_cplx *u = (so_cplx *)ud;
  zero_field(c, u);
  int ix_w = (int)lround(c->cfg.xl / lambda_x);
  int iz_w = (int)lround(c->cfg.zl / lambda_z);
  if (ix_w >= c->nx_min || iz_w >= c->nz_min || c->lu < 4) return -1;
  double c_i = omega_i / k_w;
  double amp_u = amplitude * c_i;
  double amp_T = amplitude * lapse0 / m_w;
  double r1 = k_w / m_w;
  u[W_IDX(c, iz_w, 0, ix_w, 0)] += amp_u * (-0.5 * I);
  u[W_IDX(c, iz_w, 0, ix_w, 2)] -= r1 * amp_u * (-0.5 * I);
  u[W_IDX(c, iz_w, 0, ix_w, 3)] += amp_T * (-0.5);
  u[W_IDX(c, 0, 0, 0, 0)] = uo;
  return 0;
}

/* Gaussian-enveloped internal-wave packet centred in the box: carrier wave
 * number (kx0,ky0,kz0) in box units, envelope width sigma, velocity amplitude
 * `amplitude` along y-hat x k0, temperature from the linear polarisation
 * dT/dt = -lapse w, velocity projected solenoidal, plus white-noise velocity
 * of fluctuation `noise` (reference rescale convention). */
int so_init_packet(so_ctx *c, double *ud, unsigned long long seed, int kx0, int ky0, int kz0, double sigma,
                   double amplitude, double noise) {
  so_cplx *u = (so_cplx *)ud;
  if (noise > 0.0) {
    so_init_random(c, ud, seed, 0, noise, 0, 0.0);
    if (c->lu == 4)
      for (int i = 0; i < c->nx_min; ++i)
        for (int j = 0; j < c->ny_min; ++j)
          for (int k = 0; k < c->nz_min; ++k) u[W_IDX(c, k, j, i, 3)] = 0.0;
  } else {
    zero_field(c, u);
  }
  const double qx = c->wave_x * kx0, qy = c->wave_y * ky0, qz = c->wave_z * kz0;
  /* polarisation e = y-hat x k0, normalised */
  double ex = qz, ey = 0.0, ez = -qx;
  double en = sqrt(ex * ex + ey * ey + ez * ez);
  if (en == 0.0) { ex = 0.0; ey = 0.0; ez = 1.0; en = 1.0; }
  ex /= en; ey /= en; ez /= en;
  const double q2 = qx * qx + qy * qy + qz * qz;
  const double n2 = c->cfg.buoy_fac_z * c->cfg.lapse;
  const double omega = sqrt(n2 * (qx * qx + qy * qy) / (q2 > 0 ? q2 : 1.0));
  const double vol_fac = pow(sigma * sqrt(2.0 * SO_PI), 3.0) / (c->cfg.xl * c->cfg.yl * c->cfg.zl);
  for (int i = 0; i < c->nx_min; ++i)
    for (int j = 0; j < c->ny_min; ++j)
      for (int k = 0; k < c->nz_min; ++k) {
        int ix = c->k_x[i], iy = c->k_y[j], iz = c->k_z[k];
        double sgn = ((ix + iy + iz) & 1) ? -1.0 : 1.0; /* exp(-i k.x0), x0 = box centre */
        double px = c->wave_x * (ix - kx0), py = c->wave_y * (iy - ky0), pz = c->wave_z * (iz - kz0);
        double mx = c->wave_x * (ix + kx0), my = c->wave_y * (iy + ky0), mz = c->wave_z * (iz + kz0);
        double gm = vol_fac * sgn * exp(-0.5 * sigma * sigma * (px * px + py * py + pz * pz));
        double gp = vol_fac * sgn * exp(-0.5 * sigma * sigma * (mx * mx + my * my + mz * mz));
        double re_c = 0.5 * (gm + gp);       /* transform of Re(G e^{i k0.x}) */
        so_cplx im_c = -0.5 * I * (gm - gp); /* transform of Im(G e^{i k0.x}) */
        double rkx = c->wave_x * ix, rky = c->wave_y * iy, rkz = c->wave_z * iz;
        double rk_sq = rkx * rkx + rky * rky + rkz * rkz;
        so_cplx a0 = amplitude * ex * re_c, a1 = amplitude * ey * re_c, a2 = amplitude * ez * re_c;
        if (rk_sq > 0.0) {
          so_cplx dv = (rkx * a0 + rky * a1 + rkz * a2) / rk_sq;
          a0 -= rkx * dv; a1 -= rky * dv; a2 -= rkz * dv;
        } else {
          a0 = a1 = a2 = 0.0;
        }
        u[W_IDX(c, k, j, i, 0)] += a0;
        u[W_IDX(c, k, j, i, 1)] += a1;
        u[W_IDX(c, k, j, i, 2)] += a2;
        if (c->lu == 4 && omega > 0.0) u[W_IDX(c, k, j, i, 3)] += c->cfg.lapse * amplitude * ez / omega * im_c;
      }
  enforce_symm(c, u, 0, c->lu);
  return 0;
}

/* ------------------------------------------------ raw transforms for tests */

/* one FFTPACK-convention transform of a single line: kind 0 cfftf, 1 cfftb
 * (data: n interleaved complex), 2 rfftf, 3 rfftb (data: n reals) */
int so_fft_line(int n, int kind, double *data) {
  so_cplx *work = (so_cplx *)malloc(sizeof(so_cplx) * (size_t)(2 * n + 4));
  int rc = 0;
  if (kind <= 1) {
    so_cplan p;
    if (so_cplan_init(&p, n)) { free(work); return -1; }
    if (kind == 0) so_cfftf(&p, (so_cplx *)data, work); else so_cfftb(&p, (so_cplx *)data, work);
    so_cplan_free(&p);
  } else {
    so_rplan p;
    if (so_rplan_init(&p, n)) { free(work); return -1; }
    if (kind == 2) so_rfftf(&p, data, work); else so_rfftb(&p, data, work);
    so_rplan_free(&p);
  }
  free(work);
  return rc;
}

/* ------------------------------------------------------ forcing and restart */

/* force.f:12-63 */
int so_force(so_ctx *c, double *ud, const double *ek_0, int k_force) {
  so_cplx *u = (so_cplx *)ud;
  double *work = (double *)calloc((size_t)k_force + 2, sizeof(double));
  for (int i = 0; i < c->nx_min; ++i) {
    int kx2 = c->k_x[i] * c->k_x[i];
    for (int j = 0; j < c->ny_min; ++j) {
      int k_sq2 = kx2 + c->k_y[j] * c->k_y[j];
      for (int k = 0; k < c->nz_min; ++k) {
        double factor = (i == 0 || i == c->nx2) ? 1.0 : 2.0;
        int k_sq = k_sq2 + c->k_z[k] * c->k_z[k];
        int is = (int)(sqrt((double)k_sq) + 0.5);
        if (is <= k_force) {
          double u_sq = 0.0;
          for (int n = 0; n < 3; ++n) {
            so_cplx v = u[W_IDX(c, k, j, i, n)];
            u_sq += creal(v * conj(v));
          }
          work[is] += factor * u_sq;
        }
      }
    }
  }
  double *fac = (double *)calloc((size_t)k_force + 2, sizeof(double));
  fac[0] = 1.0;
  for (int is = 1; is <= k_force; ++is) fac[is] = sqrt(ek_0[is] / work[is]);
  for (int i = 0; i < c->nx_min; ++i) {
    int kx2 = c->k_x[i] * c->k_x[i];
    for (int j = 0; j < c->ny_min; ++j) {
      int k_sq2 = kx2 + c->k_y[j] * c->k_y[j];
      for (int k = 0; k < c->nz_min; ++k) {
        int is = (int)(sqrt((double)(k_sq2 + c->k_z[k] * c->k_z[k])) + 0.5);
        if (is <= k_force)
          for (int n = 0; n < 3; ++n) u[W_IDX(c, k, j, i, n)] *= fac[is];
      }
    }
  }
  free(work);
  free(fac);
  return 0;
}

/* write_field.f:12-30: record ((n-1) Nx_min + ii-1) holds u(1:Nz_min,1:Ny_min,ii,n) */
int so_write_field(so_ctx *c, const char *fname, const double *ud) {
  const so_cplx *u = (const so_cplx *)ud;
  FILE *f = fopen(fname, "wb");
  if (!f) return -1;
  for (int n = 0; n < c->lu; ++n)
    for (int i = 0; i < c->nx_min; ++i)
      for (int j = 0; j < c->ny_min; ++j) fwrite(u + W_IDX(c, 0, j, i, n), sizeof(so_cplx), (size_t)c->nz_min, f);
  fclose(f);
  return 0;
}

/* read_field.f:37-52: size check, then the records; rows above Nz_min zeroed */
int so_read_field(so_ctx *c, const char *fname, double *ud) {
  so_cplx *u = (so_cplx *)ud;
  FILE *f = fopen(fname, "rb");
  if (!f) return -1;
  fseek(f, 0, SEEK_END);
  long found = ftell(f);
  fseek(f, 0, SEEK_SET);
  long expect = (long)sizeof(so_cplx) * c->nz_min * c->ny_min * c->nx_min * c->lu;
  if (found != expect) { fclose(f); return -2; }
  for (int n = 0; n < c->lu; ++n)
    for (int i = 0; i < c->nx_min; ++i)
      for (int j = 0; j < c->ny_min; ++j) {
        if (fread(u + W_IDX(c, 0, j, i, n), sizeof(so_cplx), (size_t)c->nz_min, f) != (size_t)c->nz_min) {
          fclose(f);
          return -3;
        }
        for (int k = c->nz_min; k < c->nze; ++k) u[W_IDX(c, k, j, i, n)] = 0;
      }
  fclose(f);
  return 0;
}

/* ------------------------------------------------------------ planes output
 * The output-step branch of sam.f:145-166 and 225-239 plus write_planes.f:
 * r(Lu+1) = p, r(Lu+2) = i kz u, r(Lu+3) = i kz v, r(Lu+4) = i kz T (stratified),
 * all transformed with u through z_trans_b, x2z_decomp and xy_trans_b into
 * uu(Nx,Ny,Nz,2 Lu) = u, v, w, [T], p, du/dz, dv/dz, [dT/dz]; the mean profile
 * of each u field (get_mean with i_remove = 0); the xy planes of all 2 Lu
 * fields (write_planes.f:34-45); the xz planes of u..p plus y_deriv of the
 * fields n != 2 (write_planes.f:56-89); the yz planes of u..p plus x_deriv of
 * the fields n != 1 (write_planes.f:105-131).  Plane indices are 1-based as
 * in the input deck.  Outputs: xy(Nx,Ny,2Lu,n_xy), xz(Nx,Nz,2Lu,n_xz),
 * yz(Ny,Nz,2Lu,n_yz), mean(Nz,Lu). */
int so_planes(so_ctx *c, const double *ud, const double *pd, const int *k_xy, int n_xy, const int *j_xz,
              int n_xz, const int *i_yz, int n_yz, double *xy, double *xz, double *yz, double *mean) {
  const so_cplx *u = (const so_cplx *)ud, *p = (const so_cplx *)pd;
  const int lu = c->lu, nu = lu, nx = c->nx, ny = c->ny, nz = c->nz, n_out = 2 * lu;
  for (int m = 0; m < n_xy; ++m) if (k_xy[m] < 1 || k_xy[m] > nz) return -1;
  for (int m = 0; m < n_xz; ++m) if (j_xz[m] < 1 || j_xz[m] > ny) return -1;
  for (int m = 0; m < n_yz; ++m) if (i_yz[m] < 1 || i_yz[m] > nx) return -1;
  const size_t nw = (size_t)c->nze * c->ny_min * c->nx_min;
  const size_t nxy = (size_t)ny * c->nx2 * nz;
  const size_t npl = (size_t)nx * ny * nz;
  so_cplx *r2 = (so_cplx *)calloc(nw * nu, sizeof(so_cplx));
  so_cplx *zb = (so_cplx *)calloc((size_t)c->ny_min * c->nx_min * c->nze * 2 * nu, sizeof(so_cplx));
  so_cplx *xyb = (so_cplx *)calloc(nxy * 2 * nu, sizeof(so_cplx));
  double *uu = (double *)malloc(sizeof(double) * npl * n_out);
  const int dz_src[3] = {0, 1, 3};
  memcpy(r2, p, sizeof(so_cplx) * nw);
  for (int f = 1; f < nu; ++f) {
    const int n = dz_src[f - 1];
    for (int i = 0; i < c->nx_min; ++i)
      for (int j = 0; j < c->ny_min; ++j)
        for (int k = 0; k < c->nz_min; ++k) {
          const double b = c->wave_z * (double)c->k_z[k];
          const so_cplx v = u[W_IDX(c, k, j, i, n)];
          r2[W_IDX(c, k, j, i, f)] = -b * cimag(v) + b * creal(v) * I;
        }
  }
  /* z_trans_b of u into blocks 0..Nu-1 and of r2 into blocks Nu..2Nu-1 */
  const size_t nzb = (size_t)c->ny_min * c->nx_min * c->nze;
  so_z_trans_b(c, (const double *)u, (double *)zb, nu);
  so_z_trans_b(c, (const double *)r2, (double *)(zb + nzb * nu), nu);
  so_x2z_decomp(c, (const double *)zb, (double *)xyb, 2 * nu);
  so_xy_trans_b(c, (double *)xyb, uu, 2 * nu);
  for (int n = 0; n < lu; ++n) {
    so_cplx *col = (so_cplx *)malloc(sizeof(so_cplx) * (size_t)c->nze);
    memcpy(col, u + W_IDX(c, 0, 0, 0, n), sizeof(so_cplx) * (size_t)c->nze);
    so_get_mean(c, (double *)col, 0, mean + (size_t)nz * n);
    free(col);
  }
  for (int m = 0; m < n_xy; ++m)
    for (int n = 0; n < n_out; ++n)
      memcpy(xy + (size_t)nx * ny * (n + (size_t)n_out * m), uu + P_IDX(c, 0, 0, k_xy[m] - 1, n),
             sizeof(double) * nx * ny);
  double *du = (double *)malloc(sizeof(double) * (size_t)nx * ny);
  for (int m = 0; m < n_xz; ++m) {
    const int j = j_xz[m] - 1;
    double *o = xz + (size_t)nx * nz * n_out * m;
    for (int n = 0; n <= lu; ++n)
      for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nx; ++i) o[i + (size_t)nx * (k + (size_t)nz * n)] = uu[P_IDX(c, i, j, k, n)];
    for (int k = 0; k < nz; ++k) {
      int L = 1;
      for (int n = 0; n < lu; ++n) {
        if (n == 1) continue;
        ++L;
        so_y_deriv(c, uu + P_IDX(c, 0, 0, k, n), du);
        for (int i = 0; i < nx; ++i) o[i + (size_t)nx * (k + (size_t)nz * (lu + L - 1))] = du[i + (size_t)nx * j];
      }
    }
  }
  for (int m = 0; m < n_yz; ++m) {
    const int i = i_yz[m] - 1;
    double *o = yz + (size_t)ny * nz * n_out * m;
    for (int n = 0; n <= lu; ++n)
      for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j) o[j + (size_t)ny * (k + (size_t)nz * n)] = uu[P_IDX(c, i, j, k, n)];
    for (int k = 0; k < nz; ++k) {
      int L = 1;
      for (int n = 0; n < lu; ++n) {
        if (n == 0) continue;
        ++L;
        so_x_deriv(c, uu + P_IDX(c, 0, 0, k, n), du);
        for (int j = 0; j < ny; ++j) o[j + (size_t)ny * (k + (size_t)nz * (lu + L - 1))] = du[i + (size_t)nx * j];
      }
    }
  }
  free(du); free(uu); free(xyb); free(zb); free(r2);
  return 0;
}

/* ------------------------------------------------ Ornstein-Uhlenbeck forcing
 * Not in the reference (force.f only clamps shell energies).  The stored
 * modes with 0 < |k| <= k_f, kx = 0 modes only in the half ky > 0 or
 * (ky = 0, kz > 0), in the order kx, ky, kz ascending; per mode three complex
 * amplitudes a with a(0) = sigma xi(0) and, after each step n,
 * u += dt P(k) a (mirror mode of kx = 0 gets the conjugate), then
 * a <- rho a + sigma sqrt(1 - rho^2) xi(n), rho = exp(-dt / T_L),
 * xi = (g1 + i g2)/sqrt(2), g1 + i g2 = sqrt(-2 ln(1 - u1)) e^{2 pi i u2}
 * (Box-Muller) with u1, u2 splitmix64 uniforms keyed by (seed, n, mode, q). */
static double so_ou_uniform(uint64_t seed, long long step, int mode, int q) {
  uint64_t ctr = ((uint64_t)step << 20) ^ ((uint64_t)mode << 4) ^ (uint64_t)q;
  uint64_t x = so_mix64(seed ^ so_mix64(ctr ^ 0xA5A5A5A5A5A5A5A5ULL));
  return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

static so_cplx so_ou_xi(uint64_t seed, long long step, int mode, int comp) {
  double u1 = 1.0 - so_ou_uniform(seed, step, mode, 2 * comp);
  double u2 = so_ou_uniform(seed, step, mode, 2 * comp + 1);
  double rad = sqrt(-2.0 * log(u1)) * 0.70710678118654752440;
  return rad * cos(2.0 * SO_PI * u2) + rad * sin(2.0 * SO_PI * u2) * I;
}

int so_set_forcing(so_ctx *c, unsigned long long seed, double k_f, double sigma, double t_l) {
  c->ou_n = 0;
  if (k_f <= 0.0 || sigma == 0.0) return 0;
  int kk = (int)floor(k_f);
  for (int kx = 0; kx <= kk; ++kx)
    for (int ky = -kk; ky <= kk; ++ky)
      for (int kz = -kk; kz <= kk; ++kz) {
        double k2 = (double)kx * kx + (double)ky * ky + (double)kz * kz;
        if (k2 == 0.0 || k2 > k_f * k_f) continue;
        if (kx == 0 && !(ky > 0 || (ky == 0 && kz > 0))) continue;
        if (kx > c->kx_max || abs(ky) > c->ky_max || abs(kz) > c->kz_max) continue;
        if (c->ou_n >= 128) return -1;
        c->ou_k[c->ou_n][0] = kx; c->ou_k[c->ou_n][1] = ky; c->ou_k[c->ou_n][2] = kz;
        ++c->ou_n;
      }
  c->ou_seed = seed; c->ou_sigma = sigma; c->ou_tl = t_l; c->ou_step = 0;
  for (int m = 0; m < c->ou_n; ++m)
    for (int q = 0; q < 3; ++q) c->ou_a[m][q] = sigma * so_ou_xi(seed, 0, m, q);
  return c->ou_n;
}

static void so_ou_apply(so_ctx *c, double *ud) {
  so_cplx *u = (so_cplx *)ud;
  const long long step = c->ou_step + 1;
  const double dt = c->dt;
  const double rho = exp(-dt / c->ou_tl), amp = c->ou_sigma * sqrt(1.0 - rho * rho);
  for (int m = 0; m < c->ou_n; ++m) {
    int kx = c->ou_k[m][0], ky = c->ou_k[m][1], kz = c->ou_k[m][2];
    double kv[3] = {c->wave_x * kx, c->wave_y * ky, c->wave_z * kz};
    double k2 = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
    so_cplx *a = c->ou_a[m];
    double dr = (kv[0] * creal(a[0]) + kv[1] * creal(a[1]) + kv[2] * creal(a[2])) / k2;
    double di = (kv[0] * cimag(a[0]) + kv[1] * cimag(a[1]) + kv[2] * cimag(a[2])) / k2;
    int j = ky >= 0 ? ky : ky + c->ny_min, k = kz >= 0 ? kz : kz + c->nz_min;
    int jm = ky > 0 ? c->ny_min - ky : -ky, km = kz > 0 ? c->nz_min - kz : -kz;
    for (int q = 0; q < 3; ++q) {
      double fr = (creal(a[q]) - kv[q] * dr) * dt, fi = (cimag(a[q]) - kv[q] * di) * dt;
      so_cplx *p = &u[W_IDX(c, k, j, kx, q)];
      *p = (creal(*p) + fr) + (cimag(*p) + fi) * I;
      if (kx == 0) {
        so_cplx *pm = &u[W_IDX(c, km, jm, 0, q)];
        *pm = (creal(*pm) + fr) + (cimag(*pm) - fi) * I;
      }
    }
    for (int q = 0; q < 3; ++q) {
      so_cplx xi = so_ou_xi(c->ou_seed, step, m, q);
      a[q] = (rho * creal(a[q]) + amp * creal(xi)) + (rho * cimag(a[q]) + amp * cimag(xi)) * I;
    }
  }
  c->ou_step = step;
}

/* ------------------------------------------------ subgrid closure coupling
 * Not in the reference: sm.f and dm.f are never linked and nothing adds an
 * eddy viscosity to rhs.f.  The coupling restated here:
 *   T_ab = u_a u_b - 2 nu_t S_ab   (the six velocity products of rhs.f:49-54)
 *   T_aT = u_a T - kappa_t dT/dx_a (the three buoyancy products)
 *   nu_t = C delta^2 |S|, |S| = sqrt(2 sum ifact S_n^2), kappa_t = nu_t / Pr_t
 * with S_ab = (i/2)(k_b u_a + k_a u_b) and dT/dx_a = i k_a T formed in wave
 * space from the stage's u (before the pre-update, like z_trans_b) and taken
 * to physical space with the same backward transforms as u.  Field m of the
 * gradient set is the one product m needs (same upper-triangle order).
 * C delta^2 is c_smag delta^2 (model 1, sm.f:32) or, for model 2, the
 * volume-averaged coefficient of dm.f evaluated at nrk = 1 of every step on
 * the physical velocity (like vel_max, rhs.f:26-28) and clipped at zero. */
static void so_les_fields(so_ctx *c, const so_cplx *u) {
  static const int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {0, 1, 1, 2, 2, 2};
  so_cplx *w = c->les_w;
  set_threads(c);
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i < c->nx_min; ++i)
    for (int j = 0; j < c->ny_min; ++j)
      for (int k = 0; k < c->nz_min; ++k) {
        const double kv[3] = {c->wave_x * c->k_x[i], c->wave_y * c->k_y[j], c->wave_z * c->k_z[k]};
        for (int m = 0; m < 6; ++m) {
          const int a = pa[m], b = pb[m];
          so_cplx v;
          if (a == b) v = I * kv[a] * u[W_IDX(c, k, j, i, a)];
          else v = 0.5 * I * (kv[b] * u[W_IDX(c, k, j, i, a)] + kv[a] * u[W_IDX(c, k, j, i, b)]);
          w[W_IDX(c, k, j, i, m)] = v;
        }
        if (c->cfg.i_strat)
          for (int a = 0; a < 3; ++a) w[W_IDX(c, k, j, i, 6 + a)] = I * kv[a] * u[W_IDX(c, k, j, i, 3)];
        if (c->les_model == 3)
          for (int a = 0; a < 3; ++a) {
            /* vorticity w_a = i (k_b u_c - k_c u_b), (a, b, c) cyclic */
            const int b = (a + 1) % 3, cc = (a + 2) % 3;
            w[W_IDX(c, k, j, i, c->lr + a)] =
                I * (kv[b] * u[W_IDX(c, k, j, i, cc)] - kv[cc] * u[W_IDX(c, k, j, i, b)]);
          }
      }
}

/* round to the nearest BF16 (ties to even) */
static float so_bf16(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  u = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
  memcpy(&x, &u, 4);
  return x;
}

/* The learned closure's 12 invariants of one point (strain S in product
 * order, temperature gradient g, vorticity w); the same formulas as the
 * CUDA feature pass (closure_invariants). */
static void so_invariants(const double *S, const double *g, const double *w, double bz, double n2, double dsq,
                          double nu, float *f) {
  const double eps = 1e-30;
  const double M[3][3] = {{S[0], S[1], S[3]}, {S[1], S[2], S[4]}, {S[3], S[4], S[5]}};
  double s2 = 0, tr3 = 0, wSw = 0, gSg = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      s2 += M[i][j] * M[i][j];
      double sq = 0;
      for (int k = 0; k < 3; ++k) sq += M[i][k] * M[k][j];
      tr3 += sq * M[j][i];
      wSw += w[i] * M[i][j] * w[j];
      gSg += g[i] * M[i][j] * g[j];
    }
  s2 = 2 * s2;
  const double sn = sqrt(s2);
  const double w2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2], wn = sqrt(w2);
  const double g2 = g[0] * g[0] + g[1] * g[1] + g[2] * g[2], gn = sqrt(g2);
  const double inv_s2 = 1.0 / (s2 + eps);
  f[0] = (float)log1p(w2 * inv_s2);
  f[1] = (float)(tr3 / (s2 * sn + eps));
  f[2] = (float)(wSw / (sn * w2 + eps));
  f[3] = (float)log1p(fabs(n2) * inv_s2);
  f[4] = (float)asinh(bz * g[2] * inv_s2);
  f[5] = (float)log1p(fabs(bz) * sqrt(g[0] * g[0] + g[1] * g[1]) * inv_s2);
  f[6] = (float)(M[2][2] / (sn + eps));
  f[7] = (float)(w[2] / (sn + wn + eps));
  f[8] = (float)(gSg / (sn * g2 + eps));
  f[9] = (float)((w[0] * g[0] + w[1] * g[1] + w[2] * g[2]) / (wn * gn + eps));
  f[10] = (float)log1p(sn * dsq / nu);
  f[11] = (float)(4 * (S[3] * S[3] + S[4] * S[4]) * inv_s2);
}

/* The network of the learned closure (12 -> 64 -> 64 -> 2, ReLU, BF16
 * weights, inputs and hidden activations): (C_nu, C_kappa) =
 * 0.02 softplus(o) in FP32 as the GPU returns them. */
static void so_mlp_eval(const float *p, const float *f, float *cout) {
  double x[12], h1[64], h2[64];
  for (int i = 0; i < 12; ++i) x[i] = so_bf16(f[i]);
  for (int n = 0; n < 64; ++n) {
    double a = 0;
    for (int i = 0; i < 12; ++i) a += (double)so_bf16(p[n * 12 + i]) * x[i];
    a += p[768 + n];
    h1[n] = so_bf16((float)(a > 0 ? a : 0));
  }
  for (int n = 0; n < 64; ++n) {
    double a = 0;
    for (int k = 0; k < 64; ++k) a += (double)so_bf16(p[832 + n * 64 + k]) * h1[k];
    a += p[4928 + n];
    h2[n] = so_bf16((float)(a > 0 ? a : 0));
  }
  for (int j = 0; j < 2; ++j) {
    double a = 0;
    for (int k = 0; k < 64; ++k) a += (double)so_bf16(p[4992 + j * 64 + k]) * h2[k];
    const float o = (float)a + p[5120 + j];
    const float sp = o > 20.f ? o : log1pf(expf(o));
    cout[j] = 0.02f * sp;
  }
}

static void so_les_stress(so_ctx *c, const double *uu, int nrk) {
  const int nx = c->nx, ny = c->ny, nz = c->nz;
  const size_t np = (size_t)nx * ny * nz;
  if (c->les_model == 2 && nrk == 1) {
    /* dm.f on the physical velocity with periodic halos */
    const size_t vol = (size_t)(nx + 2) * (ny + 2) * (nz + 2);
    for (int n = 0; n < 3; ++n) {
      double *h = c->les_uh + vol * n;
      for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
          for (int i = 0; i < nx; ++i) h[H3(c, i + 1, j + 1, k + 1)] = uu[P_IDX(c, i, j, k, n)];
      periodicity3(c, h);
    }
    const double cds = so_dm(c, c->les_uh, c->les_vt);
    c->les_cds = cds > 0.0 ? cds : 0.0; /* NaN (no strain) and backscatter give 0 */
  }
  const double cds = c->les_cds, prt_inv = c->les_prt_inv;
  double *g = c->les_g;
  if (c->les_model == 3) {
    /* the network's coefficients once per step, at stage 1, as the
     * reference's model coefficient (sam.f:128-132: cl_energy at nrk = 1);
     * stages 2 and 3 keep them and take |S| from their own strain */
    const double dsq = delta_sq_of(c), bz = c->cfg.buoy_fac_z, n2 = c->cfg.buoy_fac_z * c->cfg.lapse;
    const double nu_ref = c->cfg.vis > 1e-12 ? c->cfg.vis : 1e-12;
    const int lr = c->lr;
    float *cfs = c->les_cf;
    set_threads(c);
#pragma omp parallel for schedule(static)
    for (size_t p = 0; p < np; ++p) {
      double S[6], gt[3] = {0, 0, 0}, w[3];
      for (int m = 0; m < 6; ++m) S[m] = g[p + m * np];
      if (lr == 9)
        for (int m = 0; m < 3; ++m) gt[m] = g[p + (6 + m) * np];
      for (int m = 0; m < 3; ++m) w[m] = g[p + (lr + m) * np];
      float *cf = cfs + 2 * p;
      if (nrk == 1) {
        float f[12];
        so_invariants(S, gt, w, bz, n2, dsq, nu_ref, f);
        so_mlp_eval(c->les_mlp, f, cf);
      }
      double sum = 0.0;
      for (int m = 0; m < 6; ++m) sum += (m == 1 || m == 3 || m == 4 ? 2.0 : 1.0) * S[m] * S[m];
      const double sm = sqrt(2.0 * sum);
      const double nu = ((double)cf[0] * dsq) * sm, kap = ((double)cf[1] * dsq) * sm;
      const double nu2 = 2.0 * nu;
      for (int m = 0; m < 6; ++m) g[p + m * np] = -nu2 * g[p + m * np];
      for (int m = 6; m < lr; ++m) g[p + m * np] = -kap * g[p + m * np];
    }
    return;
  }
  set_threads(c);
#pragma omp parallel for schedule(static)
  for (size_t p = 0; p < np; ++p) {
    double sum = 0.0;
    for (int m = 0; m < 6; ++m) {
      const double s = g[p + m * np];
      sum += (m == 1 || m == 3 || m == 4 ? 2.0 : 1.0) * s * s;
    }
    const double nu = cds * sqrt(2.0 * sum);
    const double nu2 = 2.0 * nu, kap = nu * prt_inv;
    for (int m = 0; m < 6; ++m) g[p + m * np] = -nu2 * g[p + m * np];
    for (int m = 6; m < c->lr; ++m) g[p + m * np] = -kap * g[p + m * np];
  }
}

int so_set_les(so_ctx *c, int model, double c_smag, double pr_t) {
  if (model < 0 || model > 3 || !(pr_t > 0.0)) return -1;
  if (c->les_w && model == 3 && c->les_model != 3) {
    /* the learned closure carries three more fields: reallocate */
    free(c->les_w); free(c->les_zb); free(c->les_g); free(c->les_uh); free(c->les_vt); free(c->les_cf);
    c->les_w = NULL;
    c->les_cf = NULL;
  }
  c->les_model = model;
  c->les_c_smag = c_smag;
  c->les_prt_inv = 1.0 / pr_t;
  c->les_cds = model == 1 ? c_smag * delta_sq_of(c) : 0.0;
  if (!model || c->les_w) return 0;
  const int ng = c->lr + 3; /* room for the learned closure's vorticity */
  const size_t nw = (size_t)c->nze * c->ny_min * c->nx_min * ng;
  const size_t np = (size_t)c->nx * c->ny * c->nz;
  const size_t vol = (size_t)(c->nx + 2) * (c->ny + 2) * (c->nz + 2);
  c->les_w = (so_cplx *)calloc(nw, sizeof(so_cplx));
  c->les_zb = (so_cplx *)calloc((size_t)c->ny_min * c->nx_min * c->nze * ng, sizeof(so_cplx));
  c->les_g = (double *)calloc(np * ng, sizeof(double));
  c->les_cf = (float *)calloc(np * 2, sizeof(float));
  c->les_uh = (double *)calloc(vol * 3, sizeof(double));
  c->les_vt = (double *)calloc(vol, sizeof(double));
  return 0;
}

double so_les_coef(const so_ctx *c) { return c->les_cds; }

int so_mlp_set(so_ctx *c, const float *params) {
  memcpy(c->les_mlp, params, sizeof(c->les_mlp));
  return 0;
}

void so_closure_invariants(const double *S, const double *g, const double *w, double bz, double n2, double dsq,
                           double nu, float *f) {
  so_invariants(S, g, w, bz, n2, dsq, nu, f);
}
