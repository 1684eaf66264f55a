/*
 * CPU oracle for the SAM pseudo-spectral RK3 step -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C FP64 restatement of the reference's hot path, used by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker.
 * Nothing in the shipped library links or calls it.
 *
 * Arrays use the reference's own layouts (column-major Fortran, one MPI rank,
 * so nxp = Nx_min and nzp = Nze = Nz):
 *   u, r   complex (Nze, Ny_min, Nx_min, nfield)        sam.f:93
 *   uu     real    (Nx, Ny, Nz, nfield)                 sam.f:94
 *   u_sav  complex (Nz_min, Ny_min, Nx_min, 2) = (w,T)  sam.f:97
 * Complex values are interleaved (re, im) doubles.
 *
 * Pinning: the reference cannot be compiled here or on the GPU host (no
 * Fortran compiler, no MPI), so the oracle is checked against the reference's
 * own known-answer tests: FFTPACK's TFFTPK (fft.f:2838-3011), tst_transpose's
 * round trip (tst_transpose.f:124-146), the initial-divergence bound
 * (initial_field.f:144-151) and the exact plane internal-gravity-wave solution
 * of the reference's input.dat case (init.f:184-210, gw.tex:139-150).
 */
#ifndef SAM_ORACLE_H
#define SAM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Run configuration: the input.dat labels the hot path reads
 * (set_labels.f:29-102) plus the derived values initial_field.f sets. */
typedef struct so_config {
  int nx, ny, nz;
  int n_dealias; /* init.f:49-62 (0, 1, 2) */
  int i_strat;   /* 0: Lu=3/Lr=6, 1: Lu=4/Lr=9 (init.f:35-41) */
  int i_cfl;     /* vel_max.f:40-45 */
  int nrk_max;   /* 1, 2, 3 (init.f:117-145) */
  int rot_sav;   /* 1 for the tilted-box gravity wave (sam.f:176-185) */
  int i_les;     /* Chollet-Lesieur spectra (init.f:88-93, spectra.f:21) */
  int nthreads;  /* OpenMP threads (0 = runtime default) */
  double xl, yl, zl;
  double vis, pr;
  double dt0, cfl0;
  double buoy_fac_x, buoy_fac_z, lapse; /* initial_field.f:37-39,159-161 */
  double cos_theta, sin_theta;          /* initial_field.f:252-254 */
  double c_smag;                        /* sm.f:32 */
} so_config;

typedef struct so_ctx so_ctx;

so_ctx *so_create(const so_config *cfg);
void so_destroy(so_ctx *c);
/* dims: nx_min ny_min nz_min nze lu lr kx_max ky_max kz_max lm nx2 */
void so_dims(const so_ctx *c, int *out11);
void so_set_time(so_ctx *c, double time, double dt);
/* stats: time dt u_avg[4] u_var[4] u_max[4] energy cfl_x cfl_y cfl_z (18) */
void so_stats(const so_ctx *c, double *out18);

/* ---- transforms (reference layouts) ---- */
int so_z_trans_b(so_ctx *c, const double *u1, double *u2, int n_var);
int so_x2z_decomp(so_ctx *c, const double *u1, double *u2, int n_var);
int so_xy_trans_b(so_ctx *c, double *u1, double *u2, int n_var);
int so_xy_trans_f(so_ctx *c, double *u1, double *u2, int n_var);
int so_z2x_decomp(so_ctx *c, const double *u1, double *u2, int n_var);
int so_z_trans_f(so_ctx *c, double *u, int n_var);

/* ---- physics ---- */
int so_vel_max(so_ctx *c, const double *u);
int so_rhs(so_ctx *c, double *uu, double *r, const double *u_sav, int nrk);
/* one RK stage of sam.f:169-314 (no output branches) */
int so_stage(so_ctx *c, double *u, double *r, int nrk);
/* nsteps full steps (stages 1..nrk_max, then time += dt, sam.f:318) */
int so_steps(so_ctx *c, double *u, double *r, int nsteps);

/* ---- diagnostics ---- */
/* out: ek[Lm] tk[Lm] dk[Lm] vt[Lm] sample[Lm] then energy_w div_rms div_max */
int so_spectra(so_ctx *c, const double *u, const double *r, double *out);
/* out: div_avg div_rms div_max n_div */
int so_div_check(so_ctx *c, const double *u, double *out4);
double so_cl_energy(so_ctx *c, const double *u);
/* one field u(Nze,Ny_min,Nx_min); u_mean(Nze); returns jump */
double so_get_mean(so_ctx *c, double *u, int i_remove, double *u_mean);

/* ---- plane derivatives (x_deriv.f, y_deriv.f) ---- */
int so_x_deriv(so_ctx *c, const double *u, double *du);
int so_y_deriv(so_ctx *c, const double *u, double *du);

/* ---- subgrid models on haloed grids (filter.f, sm.f, dm.f) ---- */
int so_filter(so_ctx *c, const double *f_bar, double *f_hat, int n_var);
int so_sm(so_ctx *c, const double *u, double *vt);
/* returns c_delta_sq (dm.f:176) */
double so_dm(so_ctx *c, const double *u, double *vt);

/* ---- initial fields ---- */
int so_init_taylor_green(so_ctx *c, double *u);
/* random solenoidal velocity (initial_field.f:62-140 construction) with
 * spectrum kind (0: k^2, 6: k^4 exp(-2 (k/4)^2)), counter-based RNG keyed by
 * seed; then the temperature field (kind_t) when stratified; each rescaled */
int so_init_random(so_ctx *c, double *u, unsigned long long seed, int kind_u, double flct_u,
                   int kind_t, double flct_t);
/* plane internal gravity wave of the reference's i_prob=-4 case
 * (initial_field.f:225-248) */
int so_init_gw_plane(so_ctx *c, double *u, double amplitude, double lambda_x, double lambda_z,
                     double omega_i, double k_w, double m_w, double lapse0, double uo);
/* Gaussian-enveloped internal-wave packet plus white-noise velocity */
int so_init_packet(so_ctx *c, double *u, unsigned long long seed, int kx0, int ky0, int kz0,
                   double sigma, double amplitude, double noise);

/* ---- forcing and restart files ---- */
int so_force(so_ctx *c, double *u, const double *ek_0, int k_force);
/* Ornstein-Uhlenbeck forcing of 0 < |k| <= k_f applied by so_steps after
 * every step; returns the number of forced modes, -1 above 128 */
int so_set_forcing(so_ctx *c, unsigned long long seed, double k_f, double sigma, double t_l);
/* subgrid closure coupled into so_stage (not in the reference): model 0 off,
 * 1 Smagorinsky nu_t = c_smag delta^2 |S|, 2 dynamic (dm.f coefficient at
 * nrk = 1); kappa_t = nu_t / pr_t; -1 on bad arguments */
int so_set_les(so_ctx *c, int model, double c_smag, double pr_t);
double so_les_coef(const so_ctx *c);
/* model 3 of so_set_les: the learned closure; params are its 5122 FP32
 * parameters (W1 64x12, b1, W2 64x64, b2, W3 2x64, b3) */
int so_mlp_set(so_ctx *c, const float *params);
/* the closure's 12 invariants of one point */
void so_closure_invariants(const double *S, const double *g, const double *w, double bz, double n2, double dsq,
                           double nu, float *f);
int so_write_field(so_ctx *c, const char *fname, const double *u);
/* 0 ok, -1 open, -2 wrong size (read_field.f:26-32), -3 short read */
int so_read_field(so_ctx *c, const char *fname, double *u);

/* ---- planes output (sam.f:145-166, write_planes.f): u and p = r(Lu+1) in
 * wave space; 1-based plane indices; xy(Nx,Ny,2Lu,n_xy), xz(Nx,Nz,2Lu,n_xz),
 * yz(Ny,Nz,2Lu,n_yz), mean(Nz,Lu); -1 on an index out of range ---- */
int so_planes(so_ctx *c, const double *u, const double *p, const int *k_xy, int n_xy, const int *j_xz,
              int n_xz, const int *i_yz, int n_yz, double *xy, double *xz, double *yz, double *mean);

/* ---- one raw FFTPACK-convention transform (0 cfftf, 1 cfftb, 2 rfftf, 3 rfftb) ---- */
int so_fft_line(int n, int kind, double *data);

#ifdef __cplusplus
}
#endif
#endif
