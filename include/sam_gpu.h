/*
 * sam_gpu.h -- C ABI of the GB300 implementation of SAM's pseudo-spectral RK3
 * step (tslund/sam).  One process, one GPU, one context, no MPI.
 *
 * Every entry point replaces a Fortran subroutine of the reference and keeps
 * its argument list and meaning (array base addresses, n_var, isymm), so a
 * thin ISO_C_BINDING module lets sam.f call it unchanged.  Array extents come
 * from the configuration given to sam_gpu_init, just as the reference takes
 * them from its COMMON blocks (sam.h).  Arrays are HOST arrays in the
 * reference's Fortran layouts with one rank (nxp = Nx_min, nzp = Nze = Nz);
 * complex arrays are interleaved (re, im) doubles.  The same array may be
 * passed for input and output wherever the reference does so.
 *
 * All functions return 0 on success or a negative SAM_GPU_E* code; nothing
 * traps or aborts.  sam_gpu_error_string() describes the last failure.
 */
#ifndef SAM_GPU_H
#define SAM_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define SAM_GPU_OK 0
#define SAM_GPU_EINVAL -1       /* bad argument or configuration */
#define SAM_GPU_ENOTINIT -2     /* sam_gpu_init has not been called */
#define SAM_GPU_EUNSUPPORTED -3 /* a branch the reference itself cannot run */
#define SAM_GPU_ECUDA -4        /* CUDA runtime failure */
#define SAM_GPU_ENONFINITE -5   /* vel_max met NaN/Inf in the physical field */

/* sam_gpu_config.precision values */
#define SAM_GPU_PREC_FP64 64
#define SAM_GPU_PREC_DD 48
#define SAM_GPU_PREC_FP32 32

/* The input.dat values the hot path reads (set_labels.f:29-102) and the
 * derived values of init.f / initial_field.f.  Mirrors /static/, /strat/,
 * /gravity_wave/ and the RK choice of /tstep/ (sam.h:14-62). */
typedef struct sam_gpu_config {
  int nx, ny, nz;     /* Nx, Ny, Nz; Nx even */
  int n_dealias;      /* 0, 1 (2/3 rule), 2 (init.f:49-62) */
  int i_strat;        /* 0: Lu=3, Lr=6;  1: Lu=4, Lr=9 (init.f:35-41) */
  int i_cfl;          /* 1: dt from the CFL number (vel_max.f:40-45) */
  int nrk_max;        /* 1, 2 or 3 (init.f:117-145) */
  int rot_sav;        /* 1 for the tilted-box wave, i_prob = 4 (sam.f:176-185) */
  int i_les;          /* Chollet-Lesieur spectra (spectra.f:21) */
  int precision;      /* 64: FP64 drop-in; 48 (SAM_GPU_PREC_DD): the resident step
                         in double-float pairs on the FP32 pipe (about 48
                         significand bits; plain step only: no LES, forcing,
                         planes); 32: FP32 bulk with FP64 reductions.  The
                         per-routine drop-ins always compute in FP64. */
  double xl, yl, zl;  /* box */
  double vis, pr;     /* viscosity, Prandtl number */
  double dt0, cfl0;
  double buoy_fac_x, buoy_fac_z, lapse; /* initial_field.f:37-39,159-161,272-273 */
  double cos_theta, sin_theta;          /* initial_field.f:252-254 */
  double c_smag;                        /* sm.f:32 */
} sam_gpu_config;

/* /statistics/, /dynamic/ and the CFL numbers of /tstep/ (sam.h:58-77). */
typedef struct sam_gpu_stats {
  double time, dt;
  double u_avg[4], u_var[4], u_max[4];
  double energy, cfl_x, cfl_y, cfl_z;
  int nonfinite;
  int pad;
} sam_gpu_stats;

/* ---- setup (sam.f:48-62) ---- */
/* After init and fft_init (sam.f:48-51): builds the device context, the FFT
 * plans and twiddles, and allocates every device buffer the step needs. */
int sam_gpu_init(const sam_gpu_config* cfg);
int sam_gpu_finalize(void);
/* out[11]: Nx_min Ny_min Nz_min Nze Lu Lr kx_max ky_max kz_max Lm Nx/2 */
int sam_gpu_dims(int* out11);
/* /tstep/ nrk and /dynamic/ time, dt as the caller holds them (sam.h:58-62) */
int sam_gpu_set_tstep(int nrk, double dt, double time);
int sam_gpu_get_stats(sam_gpu_stats* out);
/* optional: launch on the caller's cudaStream_t (NULL = the library's own) */
int sam_gpu_set_stream(void* cuda_stream);
const char* sam_gpu_error_string(void);

/* ---- per-routine drop-ins (host arrays, reference layouts) ---- */
/* z_trans_b.f:1  u1(Nze,Ny_min,nxp,n_var) -> u2 blocks (Ny_min,nxp,Nze,n_var);
 * isymm(n_var) must be 0 (the sine/cosine branches of the reference use
 * undefined variables, z_trans_b.f:58,62,80,84). u_c, u_r, u_i are workspace and
 * may be NULL. */
int sam_gpu_z_trans_b(const double* u1, double* u2, int n_var, const int* isymm, double* u_c, double* u_r,
                      double* u_i);
/* x2z_decomp.f:1  u1 blocks (Ny_min,nxp,Nze,n_var) -> u2(Ny,Nx/2,nzp,n_var);
 * columns kx >= Nx_min of u2 are left as they were; u3 may equal u2. */
int sam_gpu_x2z_decomp(double* u1, double* u2, int n_var, double* u3);
/* xy_trans_b.f:1  complex u1(Ny,Nx/2,nzp,n_var) -> real u2(Nx,Ny,nzp,n_var);
 * u1 and u2 may be the same array. */
int sam_gpu_xy_trans_b(double* u1, double* u2, int n_var, double* work);
/* xy_trans_f.f:1  real u1(Nx,Ny,nzp,n_var) -> complex u2(nzp,Ny_min,Nx_min,n_var) */
int sam_gpu_xy_trans_f(double* u1, double* u2, int n_var, double* work);
/* z2x_decomp.f:1  with one rank the all-to-all is the identity on the
 * (nzp,Ny_min,nxp,n_var) = (Nze,Ny_min,nxp,n_var) layout; u1 and u2 may be
 * the same array, u3 is unused. */
int sam_gpu_z2x_decomp(double* u1, double* u2, int n_var, double* u3);
/* z_trans_f.f:1  in place on u(Nze,Ny_min,nxp,n_var): rows 1..Nz_min receive
 * the truncated, 1/Nz-scaled modes; rows above Nz_min are unspecified, as in
 * the reference. isymm(n_var) must be 0. */
int sam_gpu_z_trans_f(double* u, int n_var, const int* isymm, double* u_r, double* u_i);
/* vel_max.f:1  real u(Nx,Ny,nzp,Lu): updates the statistics, CFL numbers and
 * (i_cfl = 1) dt; read them with sam_gpu_get_stats. */
int sam_gpu_vel_max(const double* u, double* work);
/* rhs.f:1  uu(Nx,Ny,nzp,Lr) holds the physical u in its first Lu slots (u
 * and uu may be the same array); r(Nze,Ny_min,nxp,Lr+ipad) receives the
 * projected rhs in fields 1..Lu and the pressure in field Lu+1;
 * u_sav(Nz_min,Ny_min,nxp,3:4) is read when stratified; vel_max runs when
 * the nrk last given to sam_gpu_set_tstep is 1. */
int sam_gpu_rhs(double* u, double* uu, double* r, const double* u_sav, double* work);
/* x_deriv.f:1 / y_deriv.f:1  spectral derivative of one real (Nx,Ny) plane */
int sam_gpu_x_deriv(const double* u, double* du, double* work);
int sam_gpu_y_deriv(const double* u, double* du, double* work);

/* ---- subgrid models on haloed grids (Lx,Ly,Lz) = (Nx+2,Ny+2,Nz+2) ----
 * filter.f, sm.f and dm.f include a header the reference does not ship; the
 * symbols it would define are fixed here: periodic halo planes 1 and N+2,
 * ifact = (1,1,1,2,2,2), ip = (1,2,3,1,2,1), jp = (1,2,3,2,3,3),
 * alpha_sq = 4, delta_sq = (dx dy dz)^(2/3) (init.f:28), c_smag from the
 * configuration.  Input halos must hold the periodic images (as
 * periodicity.f sets them); outputs get periodic halos. */
/* filter.f:1  f_bar(Lx,Ly,n_var,3) -> f_hat(Lx,Ly,n_var) */
int sam_gpu_filter(const double* f_bar, double* f_hat, int n_var);
/* sm.f:1  u(Lx,Ly,Lz,3) -> vt(Lx,Ly,Lz); u_bar, s_bar are workspace (may be NULL) */
int sam_gpu_sm(const double* u, double* u_bar, double* s_bar, double* vt);
/* dm.f:1  u(Lx,Ly,Lz,3) -> vt(Lx,Ly,Lz); the work arrays may be NULL;
 * c_delta_sq (may be NULL) receives the volume-averaged coefficient that
 * dm.f:176-178 logs (times delta_sq_inv there). */
int sam_gpu_dm(const double* u, double* u_bar, double* s_bar, double* s_mag_s, double* u_bar_u_bar, double* u_hat,
               double* s_hat, double* L, double* M, double* vt, double* c_delta_sq);
/* get_mean.f:1  one field u(Nze,Ny_min,nxp): horizontal-mean profile
 * u_mean(Nze) and the linear jump; i_remove = 1 removes the jump's linear
 * profile from the kx = ky = 0 column of u in place. i_symm must be 0. */
int sam_gpu_get_mean(double* u, int i_symm, int i_remove, double* u_mean, double* jump, double* work);

/* ---- resident fused path: state stays in HBM between steps ---- */
/* after initial_field / read_field (sam.f:102-108): u(Nze,Ny_min,nxp,Lu) */
int sam_gpu_upload(const double* u);
/* r may be NULL; when given it receives (Nze,Ny_min,nxp,Lu+1): rhs + p */
int sam_gpu_download(double* u, double* r);
/* one RK stage of sam.f:169-314 on the resident state (no output branches) */
int sam_gpu_stage(int nrk);
/* nsteps steps of sam.f:122-318 (stages 1..nrk_max, then time += dt),
 * replayed from a captured CUDA graph */
int sam_gpu_step(int nsteps);

/* Measurement hook (no counterpart in the reference, which has no timers):
 * runs `reps` stages nrk on the resident state with CUDA events between the
 * five passes and returns their mean durations in ms:
 * ms5 = {z inverse, y inverse, x pass (+ vel_max), y forward, z forward+update}.
 * The state advances as in sam_gpu_stage. */
int sam_gpu_profile_stage(int nrk, int reps, float* ms5);
/* Tile and FFT-schedule autotuner (no counterpart in the reference): times
 * candidate tile sizes of each pass, and for passes along a length-256
 * dimension both FFT schedules, on the resident state (best of reps) and
 * keeps the fastest; u and r are restored afterwards.  Call after upload,
 * before stepping; results do not depend on the tiling beyond the summation
 * order of the vel_max partial sums. out6 of sam_gpu_tiles receives the
 * tiles: z-inverse rows, y-inverse columns, x-pass rows, x-pass product
 * group, y-forward planes, z-forward rows.
 * sam_gpu_set_fft_schedule / sam_gpu_fft_schedule: the FFT schedule of each
 * pass (z inverse, y inverse, x, y forward, z forward) for lines of length
 * 256: 0 the 16 x 16 register path, 1 compile-time Stockham stages of radix
 * 8, 8, 4 (other lengths have one schedule and ignore the value).  The x
 * pass also takes 2: the 16 x 16 path inside the general x-pass kernel,
 * where 0 runs the fused FP32 kernel of the plain step (same results,
 * bit for bit).  Other values are rejected (SAM_GPU_EINVAL). */
int sam_gpu_autotune(int reps);
int sam_gpu_tiles(int* out6);
/* The tiles in out6's order, set by hand instead of by the autotuner
 * (reproducible tilings); each in 1 .. 64, the x-pass rows even.  A tile
 * that does not fit a pass's shared memory is shrunk when the pass runs, as
 * the autotuner's are.  The results do not depend on the tiles beyond the
 * summation order of the vel_max partial sums. */
int sam_gpu_set_tiles(const int* in6);
int sam_gpu_set_fft_schedule(const int* sched5);
int sam_gpu_fft_schedule(int* out5);
/* Measurement hook: FP64 FMA throughput of this GPU (TFLOP/s), the ALU
 * roofline of the FP64 drop-in.  No counterpart in the reference. */
int sam_gpu_measure_fp64_peak(double* tflops);

/* ---- vel_max for callers that cannot allocate device memory ----
 * No counterpart in the reference.  For callers that own all device memory
 * through another allocator, or must not stall a step loop on cudaMalloc:
 * same sums as vel_max.f:11-34, but u_dev (real (Nx,Ny,nzp,Lu)) and
 * stats_dev (16 doubles: u_avg[4], u_var[4], u_max[4], energy, count of
 * non-finite values, 2 unused) are DEVICE pointers, and the per-plane
 * partial sums live in a 512 KB array compiled into the library (held on
 * every GPU that loads it until exit), so the call allocates nothing and needs
 * no sam_gpu_init.  nzp may not exceed SAM_GPU_NOALLOC_MAX_PLANES (else
 * SAM_GPU_EINVAL); Lu is 1..4.  The first call on each device looks up that
 * array's device address and should precede any stream capture.  Calls that
 * overlap on the GPU share the array and race.  stream: a cudaStream_t or
 * NULL for the default stream; the call is asynchronous on it. */
#define SAM_GPU_NOALLOC_MAX_PLANES 4096
int sam_gpu_vel_max_noalloc(const double* u_dev, int nx, int ny, int nzp, int lu, double* stats_dev, void* stream);

/* ---- diagnostics on the resident state ---- */
/* spectra.f:1  out[5*Lm+3]: ek tk dk vt sample, energy_w, div_rms, div_max */
int sam_gpu_spectra(double* out);
/* div_check.f:1  out[4]: div_avg div_rms div_max n_div */
int sam_gpu_div_check(double* out4);
/* cl_energy.f:1 */
int sam_gpu_cl_energy(double* e_cl);

/* force.f:1  rescale the shells 1..k_force+1 of the resident velocity back
 * to the initial shell energies ek_0 (spectra's ek of step 0) */
int sam_gpu_force(const double* ek_0, int k_force);

/* ---- planes output of the resident state ----
 * sam.f:145-166 + write_planes.f:1  at an output step (before stage 1), the
 * fields uu = u, v, w, [T], p, du/dz, dv/dz, [dT/dz] (p is the pressure the
 * last stage left, r(Lu+1)) cut into planes in write_planes' record order:
 *   xy(Nx,Ny,2Lu,n_xy)  all 2Lu fields at z = k_xy(m)      (write_planes.f:34-45)
 *   xz(Nx,Nz,2Lu,n_xz)  u..p at y = j_xz(m), then y_deriv of the fields
 *                       n = 1,3,[4]                          (write_planes.f:56-89)
 *   yz(Ny,Nz,2Lu,n_yz)  u..p at x = i_yz(m), then x_deriv of the fields
 *                       n = 2,3,[4]                          (write_planes.f:105-131)
 *   mean(Nz,Lu)         get_mean (i_remove = 0) of each u field (sam.f:161-165)
 * Plane indices are 1-based as in the input deck; at most
 * SAM_GPU_MAX_PLANES of each kind; an array may be NULL when its count is 0
 * (mean may be NULL).  The resident state is not modified. */
#define SAM_GPU_MAX_PLANES 16
int sam_gpu_planes(const int* k_xy, int n_xy, const int* j_xz, int n_xz, const int* i_yz, int n_yz, double* xy,
                   double* xz, double* yz, double* mean);

/* Ornstein-Uhlenbeck forcing (no reference counterpart; force.f only clamps
 * shell energies): the stored modes with 0 < |k| <= k_f (in units of the
 * box's fundamental wave numbers) carry three complex amplitudes each with
 * stationary rms sigma per component and correlation time t_l, advanced
 * exactly (rho = exp(-dt/t_l)) from a splitmix64 counter RNG keyed by seed;
 * every sam_gpu_step ends with u += dt P(k) a (P the solenoidal projection).
 * sam_gpu_stage does not force.  k_f <= 0 or sigma = 0 switches it off;
 * a new call restarts the amplitudes from step 0.  n_modes (may be NULL)
 * receives the number of forced modes (at most 128). */
int sam_gpu_set_forcing(unsigned long long seed, double k_f, double sigma, double t_l, int* n_modes);

/* Subgrid closure coupled into the resident step (no reference counterpart:
 * sm.f and dm.f are never linked, and rhs.f applies no eddy viscosity).
 * With a model on, every stage also takes the strain S_ab = (i/2)(k_b u_a +
 * k_a u_b) and (stratified) dT/dx_a = i k_a T to physical space and forms
 *   T_ab = u_a u_b - 2 nu_t S_ab,  T_aT = u_a T - kappa_t dT/dx_a
 * in place of rhs.f:49-57's products, nu_t = C delta^2 |S|,
 * |S| = sqrt(2 S_ab S_ab), kappa_t = nu_t / pr_t, delta^2 = (dx dy dz)^(2/3).
 *   model 0: off (the reference's products);
 *   model 1: Smagorinsky, C delta^2 = c_smag delta^2 (sm.f:32);
 *   model 2: dynamic Smagorinsky: C delta^2 is dm.f's volume-averaged
 *            coefficient (dm.f:176) of the physical velocity, evaluated at
 *            stage 1 of every step (as vel_max is, rhs.f:26-28) and clipped
 *            at zero; it starts at 0 until the first stage 1;
 *   model 3: learned closure: stage 1 of every step also takes the
 *            vorticity to physical space, forms 12 invariants of S, w and
 *            dT/dx per point (BF16) and runs the network of sam_gpu_mlp_set
 *            on the tensor cores; every stage uses the per-point (C_nu,
 *            C_kappa) of the last stage 1 with its own |S|:
 *            nu_t = C_nu delta^2 |S|, kappa_t = C_kappa delta^2 |S| (pr_t
 *            unused).  The coefficients are formed once per step like
 *            model 2's and the reference's own model coefficient
 *            (sam.f:128-132, cl_energy at nrk = 1); they are zero until the
 *            first stage 1.
 * Allocates the extra pencil, dm.f and invariant buffers on first use. */
int sam_gpu_set_les(int model, double c_smag, double pr_t);
/* C delta^2 last used (0 with the closure off) */
int sam_gpu_les_coef(double* c_delta_sq);

/* ---- learned subgrid closure (no reference counterpart) ----
 * A 12 -> 64 -> 64 -> 2 MLP (ReLU hidden layers) with BF16 weights and FP32
 * accumulation on the tensor cores (tcgen05.mma, accumulators in TMEM).
 * Its outputs are the coefficients (C_nu, C_kappa) = 0.02 softplus(o) of
 * nu_t = C_nu delta^2 |S| and kappa_t = C_kappa delta^2 |S|.  Parameters are
 * one FP32 vector of SAM_GPU_MLP_PARAMS: W1 (64 x 12, row-major [out][in]),
 * b1 (64), W2 (64 x 64), b2 (64), W3 (2 x 64), b3 (2); the network belongs to
 * the context (sam_gpu_init) and starts at zero. */
#define SAM_GPU_MLP_PARAMS 5122
#define SAM_GPU_MLP_FEATURES 12
int sam_gpu_mlp_set(const float* params, int n);
int sam_gpu_mlp_get(float* params, int n);
/* features [n][12] (host, FP32; rounded to BF16) -> coef [n][2] */
int sam_gpu_mlp_forward(const float* features, long long n, float* coef);
/* gradient of L = (1/(2n)) sum (C - target)^2 over the n points and both
 * outputs, target [n][2]; grad receives SAM_GPU_MLP_PARAMS floats, loss
 * (may be NULL) L.  The backward pass runs on the CUDA cores in FP32 with
 * the BF16 weights and activations of the forward pass. */
int sam_gpu_mlp_grad(const float* features, const float* target, long long n, float* grad, float* loss);
/* `steps` Adam steps (lr, beta 0.9/0.999, eps 1e-8) on minibatches of
 * `batch` points taken in order from the data as given (the caller
 * shuffles); loss_hist (may be NULL) receives each minibatch's loss. */
/* Backward pass of sam_gpu_mlp_grad / sam_gpu_mlp_train: 1 (default) the
 * contractions as tcgen05 tensor-core MMAs, 0 the CUDA-core kernel (the same
 * gradient to the rounding of the deltas' two-part BF16 split, about 2^-17). */
int sam_gpu_mlp_set_backward(int tensor_cores);
int sam_gpu_mlp_train(const float* features, const float* target, long long n, int steps, int batch, float lr,
                      float* loss_hist);
/* Training data of the closure.  sam_gpu_box_filter: the resident field
 * in physical space, box-filtered and downsampled by f (Nx, Ny, Nz divisible
 * by f): out(Nx/f, Ny/f, Nz/f, Lu+Lr) holds the block means of u, v, w, [T],
 * then of the products u_a u_b (rhs.f:49-54 order) and [u_a T].
 * sam_gpu_closure_inputs: the invariants the learned closure sees for the
 * resident field, feat[(z Ny + y) Nx + x][16] as BF16 bit patterns (the
 * 12 invariants, then 1.0 three times: the network's bias inputs, then 0),
 * and grads(Nx, Ny, Nz, Lr+3) the physical S (6, product order),
 * [dT/dx_a (3)] and vorticity (3) they are formed from; either may be NULL. */
int sam_gpu_box_filter(int f, double* out);
int sam_gpu_closure_inputs(unsigned short* feat, double* grads);
/* Known-answer test of the tensor-core path: d(128 x 64) = a(128 x 16)
 * b(64 x 16)^T with a, b rounded to BF16 and FP32 accumulation. */
int sam_gpu_mma_selftest(const float* a, const float* b, float* d);

/* ---- ensembles of independent runs (no reference counterpart) ----
 * sam_gpu_ensemble_create builds n contexts at once (any mix of grid sizes,
 * precisions and settings; each its own device buffers and stream) and
 * selects member 0.  While an ensemble exists, every other entry point acts
 * on the selected member (sam_gpu_ensemble_select), so members are set up
 * with the usual calls (init_*, upload, set_les, mlp_set, set_forcing,
 * autotune) and read back with download / get_stats / spectra.
 * sam_gpu_ensemble_step advances every member nsteps steps from one CUDA
 * graph per step in which each member's passes form their own branch, so
 * the small members' kernels run concurrently; it returns after the last
 * step completes.  sam_gpu_init, sam_gpu_finalize and
 * sam_gpu_ensemble_destroy end the ensemble. */
int sam_gpu_ensemble_create(const sam_gpu_config* cfgs, int n);
int sam_gpu_ensemble_select(int m);
int sam_gpu_ensemble_step(int nsteps);
int sam_gpu_ensemble_destroy(void);
/* Members in the FP32 bulk form without a subgrid closure whose transform
 * lengths are 32, 64, 96 or 128 advance together in one persistent launch per
 * RK3 stage (a ticket-ordered queue of (member, pass, tile) work items with
 * bounded dependency waits; no counterpart in the reference, which has no
 * ensembles), with at most ctas_per_sm (1, 2 or 3, the default) CTAs per SM;
 * 0 gives every member its own branch of the step graph instead.  The same
 * results either way. */
int sam_gpu_ensemble_set_persistent(int ctas_per_sm);
/* number of members the persistent launch took at the last graph build */
int sam_gpu_ensemble_persistent_members(int* n);

/* ---- restart files of the resident state ---- */
/* write_field.f:1 / read_field.f:1  vel.NNNNNN: Lu*Nx_min records of
 * Nz_min x Ny_min complex128; read_field rejects a file of the wrong size */
int sam_gpu_write_field(const char* fname);
int sam_gpu_read_field(const char* fname);
/* write_header.f:1 / read_header.f:1  header.NNNNNN: "label value" lines;
 * reading checks the restart-fixed parameters (box, grid, i_strat) against
 * the configuration, restores time and dt, and returns nt */
int sam_gpu_write_header(const char* fname, int nt);
int sam_gpu_read_header(const char* fname, int* nt);

/* ---- initial fields on the device (written to the resident state) ---- */
int sam_gpu_init_taylor_green(void);
int sam_gpu_init_random(unsigned long long seed, int kind_u, double flct_u, int kind_t, double flct_t);
int sam_gpu_init_packet(unsigned long long seed, int kx0, int ky0, int kz0, double sigma, double amplitude,
                        double noise);

#ifdef __cplusplus
}
#endif
#endif
