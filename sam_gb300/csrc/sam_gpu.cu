// Host side of the C ABI (include/sam_gpu.h): the device context that mirrors
// the reference's COMMON blocks, the FFT plans, buffer management, the
// per-routine drop-ins in the reference layouts, and the resident fused RK3
// stage with its CUDA-graph replay.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <initializer_list>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/sam_gpu.h"
#include "closure.cuh"
#include "common.cuh"
#include "diag.cuh"
#include "ens.cuh"
#include "fields.cuh"
#include "les.cuh"
#include "passes.cuh"
#include "planes.cuh"

namespace samgpu {

static char g_err[512] = "";

static int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int set_error(int code, const char* msg) { return fail(code, "%s", msg); }

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return fail(SAM_GPU_ECUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

// ---------------------------------------------------------------- FFT plans
struct Plan {
  FftPlan h{};
  FftPlan* d = nullptr;
  double2* tw64 = nullptr;
  float2* tw32 = nullptr;
  ddc* twdd = nullptr;
};

// the nearest double-float pair to an extended-precision value
static dd dd_of(long double v) {
  const float h = (float)v;
  return dd(h, (float)(v - (long double)h));
}

// Radices 8, 4, 2, 3, 5 in that order; twiddles w_{l p}^{f q} = exp(-2 pi i
// f q / (l p)) in long double, rounded once to each working precision.
static int build_plan(int n, Plan& P) {
  FftPlan& pl = P.h;
  memset(&pl, 0, sizeof(pl));
  pl.n = n;
  int r = n, ns = 0, fac[16];
  while (r % 8 == 0) { fac[ns++] = 8; r /= 8; }
  while (r % 4 == 0) { fac[ns++] = 4; r /= 4; }
  while (r % 2 == 0) { fac[ns++] = 2; r /= 2; }
  while (r % 3 == 0) { fac[ns++] = 3; r /= 3; }
  while (r % 5 == 0) { fac[ns++] = 5; r /= 5; }
  if (r != 1 || ns > 10 || n > 1024) return fail(SAM_GPU_EINVAL, "FFT length %d must be 2^a 3^b 5^c <= 1024", n);
  pl.nst = ns;
  // team width: a power of two such that no thread holds more than emax
  // values in any stage (Emax in fft_engine.cuh)
  auto team_for = [&](int emax) {
    int TW = 1;
    while (TW * emax < n) TW *= 2;
    for (;;) {
      bool ok = true;
      for (int s = 0; s < ns; ++s) {
        const int nb = n / fac[s];
        if ((nb + TW - 1) / TW > emax / fac[s]) ok = false;
      }
      if (ok) return TW;
      TW *= 2;
    }
  };
  pl.team = team_for(8);
  pl.team_sp = team_for(8);
  if (pl.team > kThreads) return fail(SAM_GPU_EINVAL, "FFT length %d needs too wide a team", n);
  std::vector<double2> t64;
  std::vector<float2> t32;
  std::vector<ddc> tdd;
  int l = 1, off = 0;
  const long double two_pi = 6.283185307179586476925286766559005768L;
  pl.tw16_off = -1;
  if (n == 256) {
    // the 16 x 16 register path (fft256_lines): w_256^{f q}, f, q in [0, 16),
    // stored q-major so the 16 threads of a team read 16 consecutive entries;
    // first in the table, so that kernels compiled for that path load only it
    pl.tw16_off = 0;
    for (int q = 0; q < 16; ++q)
      for (int f = 0; f < 16; ++f) {
        const long double a = two_pi * (long double)((f * q) % 256) / 256.0L;
        const long double c = cosl(a), sn = -sinl(a);
        t64.push_back(make_double2((double)c, (double)sn));
        t32.push_back(make_float2((float)c, (float)sn));
        tdd.push_back(ddc{dd_of(c), dd_of(sn)});
      }
    off = 256;
  }
  for (int s = 0; s < ns; ++s) {
    const int p = fac[s];
    FftStage& st = pl.st[s];
    st.p = p;
    st.l = l;
    st.m = n / (l * p);
    st.tw_off = off;
    st.mmul = (uint32_t)(((1u << 21) + (uint32_t)st.m - 1) / (uint32_t)st.m);
    for (int f = 0; f < l; ++f)
      for (int q = 1; q < p; ++q) {
        const long e = ((long)f * q) % ((long)l * p);
        const long double a = two_pi * (long double)e / (long double)(l * p);
        const long double c = cosl(a), sn = -sinl(a);
        t64.push_back(make_double2((double)c, (double)sn));
        t32.push_back(make_float2((float)c, (float)sn));
        tdd.push_back(ddc{dd_of(c), dd_of(sn)});
      }
    off += l * (p - 1);
    l *= p;
  }
  pl.tw_total = off;
  pl.tw_pass = n == 256 ? 256 : off;
  if (t64.empty()) {
    t64.push_back(make_double2(1, 0));
    t32.push_back(make_float2(1, 0));
    tdd.push_back(ddc{dd(1), dd(0)});
  }
  CK(cudaMalloc(&P.d, sizeof(FftPlan)));
  CK(cudaMemcpy(P.d, &pl, sizeof(FftPlan), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&P.tw64, sizeof(double2) * t64.size()));
  CK(cudaMemcpy(P.tw64, t64.data(), sizeof(double2) * t64.size(), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&P.tw32, sizeof(float2) * t32.size()));
  CK(cudaMemcpy(P.tw32, t32.data(), sizeof(float2) * t32.size(), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&P.twdd, sizeof(ddc) * tdd.size()));
  CK(cudaMemcpy(P.twdd, tdd.data(), sizeof(ddc) * tdd.size(), cudaMemcpyHostToDevice));
  return 0;
}

static void free_plan(Plan& P) {
  cudaFree(P.d); cudaFree(P.tw64); cudaFree(P.tw32); cudaFree(P.twdd);
  P.d = nullptr; P.tw64 = nullptr; P.tw32 = nullptr; P.twdd = nullptr;
}

template <typename T> const cx_t<T>* tw_of(const Plan& P);
template <> const double2* tw_of<double>(const Plan& P) { return P.tw64; }
template <> const float2* tw_of<float>(const Plan& P) { return P.tw32; }
template <> const ddc* tw_of<dd>(const Plan& P) { return P.twdd; }

// -------------------------------------------------------------- the context
struct Scratch {
  void* p = nullptr;
  size_t n = 0;
};

struct Ctx {
  sam_gpu_config cfg{};
  Grid g{};
  int nx2 = 0, lm = 0, k_cl = 0;
  double gamma[4] = {0, 0, 0, 0}, zeta[4] = {0, 0, 0, 0}, adv_cfl_limit = 1.0;
  int nrk = 1;
  Plan px, py, pz;
  cudaStream_t stream = nullptr, own = nullptr;
  // resident state in the working precision: U, R (lu fields), P, and the
  // pencil buffers S1 (A, then D), S2 (B), S3 (C)
  void *U = nullptr, *R = nullptr, *P = nullptr, *S1 = nullptr, *S2 = nullptr, *S3 = nullptr;
  double* partials = nullptr;
  int partial_blocks = 0;
  double* pv = nullptr;  // vel_max's wave-space sums (FP32 and double-float forms)
  dd* ift = nullptr;     // double-float form: integrating-factor tables of the stage
  DevState* state = nullptr;
  Scratch sc[4];
  // tile choices
  int ty_zi = 16, tx_yi = 16, yt_x = 8, grp_x = 9, tz_yf = 16, ty_zf = 4;
  // FFT schedule of each pass for length-256 lines (z_inv, y_inv, x, y_fwd,
  // z_fwd): 0 the 16 x 16 register path, 1 compile-time Stockham (8, 8, 4);
  // the x pass also takes 2: the register path inside the general x-pass
  // kernel even where the fused FP32 kernel applies (0 picks that one)
  int sched[5] = {0, 0, 0, 0, 0};
  OuForcing* ou = nullptr;  // device OU forcing state, null when off
  // subgrid closure coupled into the stage (sam_gpu_set_les)
  int les_model = 0;
  double les_prt_inv = 1.0, les_dxi = 0, les_dyi = 0, les_dzi = 0;
  double* les_cds = nullptr;   // device C delta^2 in use
  void* les_phys = nullptr;    // physical velocity for dm.f (3 fields, working precision)
  double* les_work = nullptr;  // dm.f work arrays
  void* les_feat = nullptr;    // learned closure: BF16 invariants [pt][16]
  float2* les_coef = nullptr;  // and its coefficients [pt]
  double les_dsq = 0;
  size_t s1_elems = 0, s2_elems = 0;
  // learned closure: FP32 parameters with Adam moments, the BF16 device form
  float *mlp_p = nullptr, *mlp_m = nullptr, *mlp_v = nullptr, *mlp_g = nullptr, *mlp_loss = nullptr;
  MlpDev* mlp_dev = nullptr;
  int* mlp_err = nullptr;
  int mlp_step = 0;
  int mlp_tc_bwd = 1;  // backward contractions on the tensor cores (else CUDA cores)
  cudaGraphExec_t gexec = nullptr;
  cudaStream_t graph_stream = nullptr;
  int graph_stale = 1;
  // set while an ensemble records this member's stage for its persistent
  // launch: the FP32 passes are recorded instead of launched
  EnsRecorder* rec = nullptr;
};

static Ctx* g_ctx = nullptr;

// Ensemble of independent contexts (sam_gpu_ensemble_*): g_ctx points at the
// selected member; the step graph runs every member on its own stream.
struct Ensemble {
  std::vector<Ctx*> members;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t gexec = nullptr;
  std::vector<cudaEvent_t> events;
  // the persistent stage launches (one per RK3 stage) over the members that
  // qualify (ens_eligible), with at most `persistent` CTAs per SM; the others
  // keep their own branches of the graph (0: every member its own branch)
  int persistent = 3;
  EnsStageLaunch stages[3];
  std::vector<EnsRecorder> recs;
  int* err = nullptr;  // a persistent launch's dependency wait timed out
  int n_persistent = 0;
};
static Ensemble* g_ens = nullptr;

static void grid_spacing(const Ctx& c, double& dxi, double& dyi, double& dzi, double& delta_sq) {
  const double dx = c.cfg.xl / c.g.nx, dy = c.cfg.yl / c.g.ny, dz = c.cfg.zl / c.g.nz;
  dxi = 1.0 / dx; dyi = 1.0 / dy; dzi = 1.0 / dz;
  delta_sq = pow(dx * dy * dz, 2.0 / 3.0);  // init.f:28
}

static int ensure(Scratch& s, size_t bytes) {
  if (s.n >= bytes) return 0;
  if (s.p) cudaFree(s.p);
  s.p = nullptr;
  s.n = 0;
  CK(cudaMalloc(&s.p, bytes));
  s.n = bytes;
  return 0;
}

static size_t csize(const Ctx& c) { return c.cfg.precision == 32 ? sizeof(float2) : sizeof(double2); }

// The resident state's working precision from / to an FP64 copy of n complex
// values (no-ops in the FP64 form, whose state is the copy).
static void state_from_fp64(Ctx& c, const double2* src, void* dst, long long n) {
  if (c.cfg.precision == 32) convert_in<float>(src, (float2*)dst, n, c.stream);
  else if (c.cfg.precision == kPrecDD) convert_in<dd>(src, (ddc*)dst, n, c.stream);
}
static void state_to_fp64(Ctx& c, const void* src, double2* dst, long long n) {
  if (c.cfg.precision == 32) convert_out<float>((const float2*)src, dst, n, c.stream);
  else if (c.cfg.precision == kPrecDD) convert_out<dd>((const ddc*)src, dst, n, c.stream);
}

static int line_ld(int n) { return line_stride(n); }

// shared memory of a tile of `lines` lines of length n plus the twiddles
// the kernel loads (schedule 1 of a length-256 pass loads the whole table)
static size_t tile_smem(const Plan& P, int lines, size_t es, int sched = 0) {
  const int ntw = sched == 1 && P.h.n == 256 ? P.h.tw_total : P.h.tw_pass;
  return es * ((size_t)ntw + (size_t)lines * line_ld(P.h.n)) + 16;
}

// dynamic shared memory budget of one CTA: the opt-in limit (227 KB on
// GB300) less room for the kernels' static shared memory
static size_t kSmemMax = 227 * 1024 - 2048;

static int pick_tile(const Plan& P, int want, int lines_per_unit, size_t es, int sched = 0) {
  int t = want;
  while (t > 1 && tile_smem(P, t * lines_per_unit, es, sched) > kSmemMax) t /= 2;
  return t;
}

// --------------------------------------------------------------- the passes
template <typename T>
static int run_z_inv(Ctx& c, const void* in, void* out, int nvar, long long in_ky, long long in_kx, long long in_n,
                     long long out_kx, long long out_z, long long out_n, int derive = 0) {
  ZInvArgs<T> a{};
  a.derive = derive;
  a.g = c.g;
  a.in = (const cx_t<T>*)in;
  a.out = (cx_t<T>*)out;
  a.tw = tw_of<T>(c.pz);
  a.nvar = nvar;
  a.sched = c.sched[0];
  a.ty = pick_tile(c.pz, c.ty_zi, 1, sizeof(cx_t<T>), a.sched);
  a.ld = line_ld(c.g.nz);
  a.in_ky = in_ky; a.in_kx = in_kx; a.in_n = in_n;
  a.out_kx = out_kx; a.out_z = out_z; a.out_n = out_n;
  const size_t smem = tile_smem(c.pz, a.ty, sizeof(cx_t<T>), a.sched);
  if constexpr (std::is_same<T, float>::value) {
    if (c.rec) {
      ens_record_z_inv(*c.rec, a, c.pz.d, smem);
      return 0;
    }
  }
  launch_z_inv<T>(a, c.pz.d, smem, c.stream);
  return 0;
}

template <typename T>
static int run_y_inv(Ctx& c, const void* in, void* out, int nvar, int in_full, long long in_kx, long long in_z,
                     long long in_n, long long out_y, long long out_z, long long out_n) {
  YInvArgs<T> a{};
  a.g = c.g;
  a.in = (const cx_t<T>*)in;
  a.out = (cx_t<T>*)out;
  a.tw = tw_of<T>(c.py);
  a.nvar = nvar;
  a.sched = c.sched[1];
  a.tx = pick_tile(c.py, c.tx_yi, 1, sizeof(cx_t<T>), a.sched);
  a.ld = line_ld(c.g.ny);
  a.in_full = in_full;
  a.in_kx = in_kx; a.in_z = in_z; a.in_n = in_n;
  a.out_y = out_y; a.out_z = out_z; a.out_n = out_n;
  const size_t smem = tile_smem(c.py, a.tx, sizeof(cx_t<T>), a.sched);
  if constexpr (std::is_same<T, float>::value) {
    if (c.rec) {
      ens_record_y_inv(*c.rec, a, c.py.d, smem);
      return 0;
    }
  }
  launch_y_inv<T>(a, c.py.d, smem, c.stream);
  return 0;
}

// whether the x pass runs the 16 x 16 register path
static bool x_reg16(const Ctx& c) { return c.g.nx == 256 && c.sched[2] != 1; }

// lines the reduction scratch of vel_max occupies (FP64 partials of each warp)
template <typename T>
static int x_red_lines(const Ctx& c) {
  const size_t red = sizeof(double) * 4 * (x_threads((int)sizeof(T), x_reg16(c)) / 32) + 64;
  const size_t line = sizeof(cx_t<T>) * (size_t)line_ld(c.g.nx);
  return (int)((red + line - 1) / line);
}

// x pass tile: yt rows (yt/2 input lines per field) and `grp` product lines
// per round of out_mode 2.  c.grp_x caps the round at that many product
// fields; the round then takes as many lines as fit, in whole rounds of the
// CTA's teams where it exceeds them.  vel_max's reduction scratch shares the
// product lines' space (at least x_red_lines lines are allocated).
template <typename T>
static int x_tile(Ctx& c, int nin, int out_mode, int& yt, int& grp) {
  const size_t es = sizeof(cx_t<T>);
  const int threads = x_threads((int)sizeof(T), x_reg16(c));
  const int team = x_reg16(c) ? 16 : (sizeof(T) == 4 ? c.px.h.team_sp : c.px.h.team);
  const int teams = threads / team > 0 ? threads / team : 1;
  // FP32 tiles leave room for three CTAs per SM (72 registers each; two
  // CTAs with 16-row tiles measured slower), FP64 tiles for two (up to 128
  // registers each): the FP64 pipe needs the second CTA's warps to cover its
  // dependency latency
  const size_t budget = sizeof(T) == 4 ? kSmemMax / 3 - 1024 : kSmemMax / 2 - 1024;
  const size_t line = es * (size_t)line_ld(c.g.nx);
  const size_t rmin = line * (size_t)x_red_lines<T>(c);
  for (yt = c.yt_x;; yt /= 2) {
    const int yp = yt / 2;
    const size_t base = tile_smem(c.px, nin * yp, es, c.sched[2]);
    if (out_mode != 2) {
      grp = 0;
      if (base + rmin <= budget) return 0;
    } else if (base + rmin <= budget) {
      const int fit = (int)((budget - base) / line);
      const int total = c.g.lr * yp;
      grp = std::min(std::min(fit, std::max(c.grp_x, 1) * yp), total);
      if (grp > teams && grp < total) grp -= grp % teams;
      return 0;
    }
    if (yt <= 2) return fail(SAM_GPU_EINVAL, "x pass does not fit in shared memory (Nx=%d)", c.g.nx);
  }
}

template <typename T>
static size_t x_smem(Ctx& c, int nin, int yt, int grp) {
  return tile_smem(c.px, nin * (yt / 2) + std::max(grp, x_red_lines<T>(c)), sizeof(cx_t<T>), c.sched[2]);
}

template <typename T>
static int run_x_pass(Ctx& c, int in_mode, int out_mode, int nin, const void* in, const void* in_phys,
                      long long in_y, long long in_z, long long in_n, void* out, void* out_phys, long long out_kx,
                      long long out_z, long long out_n, long long out_py, long long out_pz, long long out_pn,
                      bool stats, int les = 0) {
  XPassArgs<T> a{};
  if (les) {
    a.les = les;
    a.les_cds = c.les_cds;
    a.les_prt_inv = c.les_prt_inv;
    a.les_coef = c.les_coef;
    a.les_dsq = c.les_dsq;
  }
  if (out_mode == 4) {
    a.feat = c.les_feat;
    a.f_bz = c.cfg.buoy_fac_z;
    a.f_n2 = c.cfg.buoy_fac_z * c.cfg.lapse;
    a.f_dsq = c.les_dsq;
    a.f_nu = c.cfg.vis > 1e-12 ? c.cfg.vis : 1e-12;
  }
  a.g = c.g;
  a.in = (const cx_t<T>*)in;
  a.in_phys = (const T*)in_phys;
  a.out = (cx_t<T>*)out;
  a.out_phys = (T*)out_phys;
  a.tw = tw_of<T>(c.px);
  a.in_mode = in_mode;
  a.out_mode = out_mode;
  a.nin = nin;
  a.sched = c.sched[2];
  int rc = x_tile<T>(c, nin, out_mode, a.yt, a.group);
  if (rc) return rc;
  a.ld = line_ld(c.g.nx);
  a.in_y = in_y; a.in_z = in_z; a.in_n = in_n;
  a.out_kx = out_kx; a.out_z = out_z; a.out_n = out_n;
  a.out_py = out_py; a.out_pz = out_pz; a.out_pn = out_pn;
  a.partials = nullptr;
  const int nblk = x_pass_blocks<T>(a);
  if (stats) {
    if (nblk > c.partial_blocks) {
      cudaFree(c.partials);
      c.partials = nullptr;
      CK(cudaMalloc(&c.partials, sizeof(double) * 4 * 4 * (size_t)nblk));
      c.partial_blocks = nblk;
    }
    a.partials = c.partials;
    // the FP32 and double-float forms take vel_max's sums from wave space
    // (Parseval, FP64 arithmetic): the x pass then only forms max |u| and
    // the NaN check
    a.max_only = (sizeof(T) == 4 || kIsDD<T>) && in_mode == 0 && in == c.S2;
    a.vmax = reinterpret_cast<int*>(c.pv + 4 * ((size_t)kParsevalBlocks + 1));
  }
  if constexpr (std::is_same<T, float>::value) {
    if (c.rec) {
      EnsParsevalArgs pa{(const float2*)c.U, c.g, c.pv};
      EnsFinishArgs fa{c.partials, nblk, c.g, c.state, c.cfg.i_cfl, c.cfg.cfl0, c.adv_cfl_limit, c.pv,
                       kParsevalBlocks, a.vmax};
      if (stats && !a.max_only) return fail(SAM_GPU_EUNSUPPORTED, "ensemble stage: FP64 vel_max partials");
      ens_record_x_pass(*c.rec, a, c.px.d, x_smem<T>(c, nin, a.yt, a.group), stats, &pa, &fa);
      return 0;
    }
  }
  launch_x_pass<T>(a, c.px.d, x_smem<T>(c, nin, a.yt, a.group), c.stream);
  if (stats) {
    if (a.max_only) launch_parseval<T>((const cx_t<T>*)c.U, c.g, c.pv, c.stream);
    launch_vel_max_finish(c.partials, nblk, c.g, c.state, c.cfg.i_cfl, c.cfg.cfl0, c.adv_cfl_limit, c.stream,
                          a.max_only ? c.pv : nullptr, kParsevalBlocks, a.vmax, kIsDD<T> ? 1 : 0);
  }
  return 0;
}

template <typename T>
static int run_y_fwd(Ctx& c, const void* in, void* out, int nvar, long long in_kx, long long in_z, long long in_n,
                     long long out_ky, long long out_kx, long long out_n) {
  YFwdArgs<T> a{};
  a.g = c.g;
  a.in = (const cx_t<T>*)in;
  a.out = (cx_t<T>*)out;
  a.tw = tw_of<T>(c.py);
  a.nvar = nvar;
  a.sched = c.sched[3];
  a.tz = pick_tile(c.py, c.tz_yf, 1, sizeof(cx_t<T>), a.sched);
  a.ld = line_ld(c.g.ny);
  a.in_kx = in_kx; a.in_z = in_z; a.in_n = in_n;
  a.out_ky = out_ky; a.out_kx = out_kx; a.out_n = out_n;
  const size_t smem = tile_smem(c.py, a.tz, sizeof(cx_t<T>), a.sched);
  if constexpr (std::is_same<T, float>::value) {
    if (c.rec) {
      ens_record_y_fwd(*c.rec, a, c.py.d, smem);
      return 0;
    }
  }
  launch_y_fwd<T>(a, c.py.d, smem, c.stream);
  return 0;
}

static StageConsts stage_consts(const Ctx& c, int nrk, int write_p) {
  StageConsts s{};
  s.nrk = nrk;
  s.last = nrk == c.cfg.nrk_max;
  s.i_strat = c.cfg.i_strat;
  s.rot_sav = c.cfg.rot_sav;
  s.i_cfl = c.cfg.i_cfl;
  s.write_p = write_p;
  s.gamma = c.gamma[nrk - 1];
  s.zeta = c.zeta[nrk - 1];
  s.vis = c.cfg.vis;
  s.pr_inv = 1.0 / c.cfg.pr;
  s.buoy_fac_x = c.cfg.buoy_fac_x;
  s.buoy_fac_z = c.cfg.buoy_fac_z;
  s.lapse = c.cfg.lapse;
  s.cos_theta = c.cfg.cos_theta;
  s.sin_theta = c.cfg.sin_theta;
  s.cfl0 = c.cfg.cfl0;
  s.adv_cfl_limit = c.adv_cfl_limit;
  return s;
}

template <typename T>
static int run_z_fwd(Ctx& c, ZFwdArgs<T>& a) {
  a.g = c.g;
  a.tw = tw_of<T>(c.pz);
  a.ld = line_ld(c.g.nz);
  a.sched = c.sched[4];
  a.ty = pick_tile(c.pz, c.ty_zf, a.nf, sizeof(cx_t<T>), a.sched);
  if (kIsDD<T> && a.mode == 2) {
    launch_if_tables(c.state, a.sc, c.g, c.ift, c.stream);
    a.ift = c.ift;
  }
  const size_t smem = tile_smem(c.pz, a.ty * a.nf, sizeof(cx_t<T>), a.sched);
  if constexpr (std::is_same<T, float>::value) {
    if (c.rec) {
      ens_record_z_fwd(*c.rec, a, c.pz.d, smem);
      return 0;
    }
  }
  launch_z_fwd<T>(a, c.pz.d, smem, c.stream);
  return 0;
}

// One fused RK stage on the resident state (sam.f:169-314).  When ev is
// given, ev[p] is recorded before pass p and ev[5] after the last pass; when
// only >= 0, just pass `only` (0..4) runs (used by the autotuner).
template <typename T>
static int enqueue_stage(Ctx& c, int nrk, cudaEvent_t* ev = nullptr, int only = -1) {
  const Grid& g = c.g;
  const long long nzmm = (long long)g.mx * g.my * g.mz;
  int rc = 0;
  auto run = [&](int p) { return only < 0 || only == p; };
  // with a subgrid closure the backward transforms also carry the Lr
  // gradient fields the products need
  const bool les = c.les_model != 0;
  const int nin = g.lu + (les ? g.lr : 0);
  // the learned closure's coefficients are formed once per step, at stage
  // 1, like the reference's model coefficient (sam.f:128-132: cl_energy at
  // nrk = 1) and dm.f's here; stages 2 and 3 keep them and take |S| from
  // their own strain
  const bool coef_stage = c.les_model == 3 && nrk == 1;
  const int ninv = nin + (coef_stage ? 3 : 0);  // + vorticity for the invariants
  if (ev) cudaEventRecord(ev[0], c.stream);
  // z inverse: U(n, kx, ky, kz) -> A(n, z, kx, ky)
  if (run(0))
    rc = run_z_inv<T>(c, c.U, c.S1, ninv, g.mz, (long long)g.my * g.mz, nzmm, g.my, (long long)g.mx * g.my,
                      (long long)g.nz * g.mx * g.my, les ? 1 : 0);
  if (rc) return rc;
  if (ev) cudaEventRecord(ev[1], c.stream);
  // y inverse: A -> B(n, z, y, kx)
  if (run(1))
    rc = run_y_inv<T>(c, c.S1, c.S2, ninv, 0, g.my, (long long)g.mx * g.my, (long long)g.nz * g.mx * g.my, g.mx,
                      (long long)g.ny * g.mx, (long long)g.nz * g.ny * g.mx);
  if (rc) return rc;
  if (ev) cudaEventRecord(ev[2], c.stream);
  // dynamic closure at nrk = 1 (once per step, like vel_max): the physical
  // velocity, then dm.f's coefficient on it
  if constexpr (!kIsDD<T>) {  // (the double-float form has no closure)
    if (run(2) && c.les_model == 2 && nrk == 1) {
      rc = run_x_pass<T>(c, 0, 0, 3, c.S2, nullptr, g.mx, (long long)g.ny * g.mx, (long long)g.nz * g.ny * g.mx,
                         nullptr, c.les_phys, 0, 0, 0, g.nx, (long long)g.nx * g.ny, (long long)g.nx * g.ny * g.nz,
                         false);
      if (rc) return rc;
      les_dynamic<T>((const T*)c.les_phys, c.les_work, c.les_cds, g.nx, g.ny, g.nz, c.les_dxi, c.les_dyi, c.les_dzi,
                     c.stream);
    }
  }
  // learned closure: the invariants of every point, then the network
  if (run(2) && coef_stage) {
    const long long bn = (long long)g.nz * g.ny * g.mx;
    rc = run_x_pass<T>(c, 0, 4, g.lr + 3, (const cx_t<T>*)c.S2 + g.lu * bn, nullptr, g.mx, (long long)g.ny * g.mx,
                       bn, nullptr, nullptr, 0, 0, 0, 0, 0, 0, false);
    if (rc) return rc;
    if (mlp_forward((const __nv_bfloat16*)c.les_feat, (long long)g.nx * g.ny * g.nz, c.mlp_dev, c.les_coef,
                    nullptr, c.mlp_err, c.stream) < 0)
      return fail(SAM_GPU_ECUDA, "closure network: no TMA tensor map (cuTensorMapEncodeTiled unavailable)");
  }
  // x pass: B -> C(m, z, kx, y) with vel_max at nrk = 1
  if (run(2))
    rc = run_x_pass<T>(c, 0, 2, nin, c.S2, nullptr, g.mx, (long long)g.ny * g.mx, (long long)g.nz * g.ny * g.mx,
                       c.S3, nullptr, g.ny, (long long)g.mx * g.ny, (long long)g.nz * g.mx * g.ny, 0, 0, 0, nrk == 1,
                       c.les_model == 3 ? 2 : (les ? 1 : 0));
  if (rc) return rc;
  if (ev) cudaEventRecord(ev[3], c.stream);
  // y forward: C -> D(m, kx, ky, z)
  if (run(3))
    rc = run_y_fwd<T>(c, c.S3, c.S1, g.lr, g.ny, (long long)g.mx * g.ny, (long long)g.nz * g.mx * g.ny, g.nz,
                      (long long)g.my * g.nz, (long long)g.mx * g.my * g.nz);
  if (rc) return rc;
  if (ev) cudaEventRecord(ev[4], c.stream);
  if (!run(4)) {
    if (ev) cudaEventRecord(ev[5], c.stream);
    return 0;
  }
  // z forward + rhs + RK update
  ZFwdArgs<T> a{};
  a.in = (cx_t<T>*)c.S1;
  a.mode = 2;
  a.nf = g.lr;
  a.in_ky = g.nz; a.in_kx = (long long)g.my * g.nz; a.in_n = (long long)g.mx * g.my * g.nz;
  a.u = (cx_t<T>*)c.U;
  a.r = (cx_t<T>*)c.R;
  a.p = (cx_t<T>*)c.P;
  a.u_ky = g.mz; a.u_kx = (long long)g.my * g.mz; a.u_n = nzmm;
  a.state = c.state;
  a.sc = stage_consts(c, nrk, 1);
  rc = run_z_fwd<T>(c, a);
  if (ev) cudaEventRecord(ev[5], c.stream);
  return rc;
}

static int stage_any(Ctx& c, int nrk, cudaEvent_t* ev = nullptr, int only = -1) {
  if (c.cfg.precision == 32) return enqueue_stage<float>(c, nrk, ev, only);
  if (c.cfg.precision == kPrecDD) return enqueue_stage<dd>(c, nrk, ev, only);
  return enqueue_stage<double>(c, nrk, ev, only);
}

static int check_launch() {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(SAM_GPU_ECUDA, "kernel launch: %s", cudaGetErrorString(e));
  return 0;
}

static int sync_stream(Ctx& c) {
  CK(cudaStreamSynchronize(c.stream));
  return check_launch();
}

static void free_ctx(Ctx* c) {
  if (!c) return;
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  free_plan(c->px); free_plan(c->py); free_plan(c->pz);
  cudaFree(c->U); cudaFree(c->R); cudaFree(c->P);
  cudaFree(c->S1); cudaFree(c->S2); cudaFree(c->S3);
  cudaFree(c->partials); cudaFree(c->state); cudaFree(c->ou); cudaFree(c->pv); cudaFree(c->ift);
  cudaFree(c->les_cds); cudaFree(c->les_phys); cudaFree(c->les_work);
  cudaFree(c->les_feat); cudaFree(c->les_coef);
  cudaFree(c->mlp_p); cudaFree(c->mlp_m); cudaFree(c->mlp_v); cudaFree(c->mlp_g); cudaFree(c->mlp_loss);
  cudaFree(c->mlp_dev); cudaFree(c->mlp_err);
  for (auto& s : c->sc) cudaFree(s.p);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
}

// Planes output (sam.f:145-166, write_planes.f) on the resident state: the
// batch u, p, i kz (u, v, [T]), then i ky (u, w, [T]) when xz planes are asked
// for and i kx (v, w, [T]) when yz planes are, through the inverse passes into
// physical space, then the plane cuts.  Scratch: sc[0] holds the wave batch,
// then the physical batch; sc[1] the z-inverse blocks, then the planes; sc[2]
// the y-inverse blocks; sc[3] the mean columns.
template <typename T>
static int planes_impl(Ctx& c, const PlaneSel& sel0, double* xy, double* xz, double* yz, double* mean) {
  using Cx = cx_t<T>;
  const Grid& g = c.g;
  const int lu = g.lu;
  PlaneFields pf{};
  PlaneSel sel = sel0;
  int nf = 0;
  auto add = [&](int src, int op) {
    pf.src[nf] = src;
    pf.op[nf] = op;
    return nf++;
  };
  // the fields write_planes differentiates: z (sam.f:152-157), y (write_planes.f:79-86: n != 2),
  // x (write_planes.f:119-126: n != 1), as 0-based field numbers
  const int dz_src[3] = {0, 1, 3}, dy_src[3] = {0, 2, 3}, dx_src[3] = {1, 2, 3};
  for (int n = 0; n < lu; ++n) add(n, 0);
  add(-1, 0);
  for (int m = 0; m < lu - 1; ++m) add(dz_src[m], 1);
  for (int s = 0; s < 2 * lu; ++s) sel.fxy[s] = s;
  if (sel.n_xz > 0) {
    for (int s = 0; s <= lu; ++s) sel.fxz[s] = s;
    for (int m = 0; m < lu - 1; ++m) sel.fxz[lu + 1 + m] = add(dy_src[m], 2);
  }
  if (sel.n_yz > 0) {
    for (int s = 0; s <= lu; ++s) sel.fyz[s] = s;
    for (int m = 0; m < lu - 1; ++m) sel.fyz[lu + 1 + m] = add(dx_src[m], 3);
  }
  pf.nf = nf;
  sel.n_out = 2 * lu;
  const size_t nm = (size_t)g.mx * g.my * g.mz;
  const size_t vol = (size_t)g.nx * g.ny * g.nz;
  const size_t n_planes = ((size_t)sel.n_xy * g.nx * g.ny + (size_t)sel.n_xz * g.nx * g.nz +
                           (size_t)sel.n_yz * g.ny * g.nz) * sel.n_out;
  const size_t w_bytes = nm * nf * sizeof(Cx), ph_bytes = vol * nf * sizeof(T);
  const size_t a_bytes = (size_t)nf * g.nz * g.mx * g.my * sizeof(Cx);
  const size_t b_bytes = (size_t)nf * g.nz * g.ny * g.mx * sizeof(Cx);
  int rc;
  if ((rc = ensure(c.sc[0], w_bytes > ph_bytes ? w_bytes : ph_bytes)) ||
      (rc = ensure(c.sc[1], a_bytes > n_planes * 8 ? a_bytes : n_planes * 8)) || (rc = ensure(c.sc[2], b_bytes)) ||
      (rc = ensure(c.sc[3], ((size_t)g.mz * 2 + (size_t)g.nz * lu + 8) * 8)))
    return rc;
  planes_fields<T>(g, pf, (const Cx*)c.U, (const Cx*)c.P, (Cx*)c.sc[0].p, c.stream);
  if ((rc = run_z_inv<T>(c, c.sc[0].p, c.sc[1].p, nf, g.mz, (long long)g.my * g.mz, (long long)nm, g.my,
                         (long long)g.mx * g.my, (long long)g.nz * g.mx * g.my)))
    return rc;
  if ((rc = run_y_inv<T>(c, c.sc[1].p, c.sc[2].p, nf, 0, g.my, (long long)g.mx * g.my,
                         (long long)g.nz * g.mx * g.my, g.mx, (long long)g.ny * g.mx,
                         (long long)g.nz * g.ny * g.mx)))
    return rc;
  if ((rc = run_x_pass<T>(c, 0, 0, nf, c.sc[2].p, nullptr, g.mx, (long long)g.ny * g.mx,
                          (long long)g.nz * g.ny * g.mx, nullptr, c.sc[0].p, 0, 0, 0, g.nx, (long long)g.nx * g.ny,
                          (long long)vol, false)))
    return rc;
  double* d_xy = (double*)c.sc[1].p;
  double* d_xz = d_xy + (size_t)sel.n_xy * sel.n_out * g.nx * g.ny;
  double* d_yz = d_xz + (size_t)sel.n_xz * sel.n_out * g.nx * g.nz;
  planes_gather<T>(g, sel, (const T*)c.sc[0].p, d_xy, d_xz, d_yz, c.stream);
  if (mean) {
    double2* col = (double2*)c.sc[3].p;
    double* dmean = (double*)(col + g.mz);
    double* djump = dmean + (size_t)g.nz * lu;
    for (int n = 0; n < lu; ++n) {
      convert_out<T>((const Cx*)c.U + (size_t)n * nm, col, g.mz, c.stream);
      les_get_mean(col, g.mz, g.kz, g.nz, 0, c.pz.d, c.pz.tw64, c.pz.h, dmean + (size_t)n * g.nz, djump, c.stream);
    }
    CK(cudaMemcpyAsync(mean, dmean, (size_t)g.nz * lu * 8, cudaMemcpyDeviceToHost, c.stream));
  }
  if (sel.n_xy)
    CK(cudaMemcpyAsync(xy, d_xy, (size_t)sel.n_xy * sel.n_out * g.nx * g.ny * 8, cudaMemcpyDeviceToHost, c.stream));
  if (sel.n_xz)
    CK(cudaMemcpyAsync(xz, d_xz, (size_t)sel.n_xz * sel.n_out * g.nx * g.nz * 8, cudaMemcpyDeviceToHost, c.stream));
  if (sel.n_yz)
    CK(cudaMemcpyAsync(yz, d_yz, (size_t)sel.n_yz * sel.n_out * g.ny * g.nz * 8, cudaMemcpyDeviceToHost, c.stream));
  return 0;
}

}  // namespace samgpu

using namespace samgpu;

#define NEED_CTX()                                                         \
  if (!g_ctx) return fail(SAM_GPU_ENOTINIT, "sam_gpu_init has not been called"); \
  Ctx& c = *g_ctx

extern "C" {

const char* sam_gpu_error_string(void) { return g_err; }

static int init_ctx(const sam_gpu_config* cfg);
static void ensemble_free();

int sam_gpu_init(const sam_gpu_config* cfg) {
  if (g_ens) ensemble_free();
  if (g_ctx) { free_ctx(g_ctx); g_ctx = nullptr; }
  return init_ctx(cfg);
}

static int init_ctx(const sam_gpu_config* cfg) {
  if (!cfg) return fail(SAM_GPU_EINVAL, "null config");
  if (cfg->nx < 2 || cfg->nx % 2 || cfg->ny < 1 || cfg->nz < 1)
    return fail(SAM_GPU_EINVAL, "grid %d x %d x %d: Nx must be even and >= 2", cfg->nx, cfg->ny, cfg->nz);
  if (cfg->precision != 64 && cfg->precision != 32 && cfg->precision != kPrecDD)
    return fail(SAM_GPU_EINVAL, "precision must be 64, 48 (double-float pairs) or 32");
  if (cfg->nrk_max < 1 || cfg->nrk_max > 3) return fail(SAM_GPU_EINVAL, "nrk_max must be 1, 2 or 3");
  Ctx* c = new Ctx();
  c->cfg = *cfg;
  Grid& g = c->g;
  g.nx = cfg->nx; g.ny = cfg->ny; g.nz = cfg->nz; g.nze = cfg->nz;
  // init.f:49-73
  switch (cfg->n_dealias) {
    case 0: g.kx = g.nx / 2 - 1; g.ky = g.ny / 2 - 1; g.kz = g.nz / 2 - 1; break;
    case 2:
      g.kx = g.nx / 2 - 1;
      g.ky = (int)(((double)g.ny - 0.1) / 3.0);
      g.kz = (int)(((double)g.nz - 0.1) / 3.0);
      break;
    default:
      g.kx = (int)(((double)g.nx - 0.1) / 3.0);
      g.ky = (int)(((double)g.ny - 0.1) / 3.0);
      g.kz = (int)(((double)g.nz - 0.1) / 3.0);
  }
  if (g.ky < 0) g.ky = 0;
  if (g.kz < 0) g.kz = 0;
  g.mx = g.kx + 1; g.my = 2 * g.ky + 1; g.mz = 2 * g.kz + 1;
  g.lu = cfg->i_strat ? 4 : 3;
  g.lr = cfg->i_strat ? 9 : 6;
  const double pi = 3.14159265358979323846;
  g.wave_x = 2.0 * pi / cfg->xl;
  g.wave_y = 2.0 * pi / cfg->yl;
  g.wave_z = 2.0 * pi / cfg->zl;
  c->nx2 = g.nx / 2;
  const int ksq = g.kx * g.kx + g.ky * g.ky + g.kz * g.kz;
  c->lm = (int)(sqrt((double)ksq) + 0.5) + 1;
  c->k_cl = (int)(g.nx / 3.0);
  // init.f:117-145
  if (cfg->nrk_max == 1) {
    c->gamma[0] = 1.0; c->adv_cfl_limit = 1.0;
  } else if (cfg->nrk_max == 2) {
    c->gamma[0] = 1.0; c->gamma[1] = 0.5; c->zeta[1] = -0.5; c->adv_cfl_limit = 1.0;
  } else {
    c->gamma[0] = 8.0 / 15.0; c->gamma[1] = 5.0 / 12.0; c->gamma[2] = 3.0 / 4.0;
    c->zeta[1] = -17.0 / 60.0; c->zeta[2] = -5.0 / 12.0;
    c->adv_cfl_limit = sqrt(3.0);
  }
  g_ctx = c;
  int rc;
  if ((rc = build_plan(g.nx, c->px)) || (rc = build_plan(g.ny, c->py)) || (rc = build_plan(g.nz, c->pz))) {
    free_ctx(c); g_ctx = nullptr; return rc;
  }
  cudaError_t e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
  if (e != cudaSuccess) { free_ctx(c); g_ctx = nullptr; return fail(SAM_GPU_ECUDA, "stream: %s", cudaGetErrorString(e)); }
  c->stream = c->own;
  {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess && optin > 4096)
      kSmemMax = (size_t)optin - 2048;
  }
  set_smem_limits<double>();
  set_smem_limits<float>();
  set_smem_limits<dd>();
  diag_set_smem_limits();
  const size_t es = csize(*c);
  const size_t nzmm = (size_t)g.mx * g.my * g.mz;
  const size_t s1 = (size_t)g.lr * g.mx * g.my * g.nz;
  const size_t s2 = (size_t)g.lu * g.nz * g.ny * g.mx;
  c->s1_elems = s1;
  c->s2_elems = s2;
  const size_t s3 = (size_t)g.lr * g.nz * g.mx * g.ny;
  bool ok = cudaMalloc(&c->U, es * g.lu * nzmm) == cudaSuccess && cudaMalloc(&c->R, es * g.lu * nzmm) == cudaSuccess &&
            cudaMalloc(&c->P, es * nzmm) == cudaSuccess && cudaMalloc(&c->S1, es * s1) == cudaSuccess &&
            cudaMalloc(&c->S2, es * s2) == cudaSuccess && cudaMalloc(&c->S3, es * s3) == cudaSuccess &&
            cudaMalloc(&c->state, sizeof(DevState)) == cudaSuccess;
  // vel_max partials for any x-pass tiling (at least one row per CTA), so no
  // allocation ever happens inside a captured step
  c->partial_blocks = g.nz * g.ny;
  ok = ok && cudaMalloc(&c->partials, sizeof(double) * 4 * 4 * (size_t)c->partial_blocks) == cudaSuccess;
  const size_t pv_bytes = sizeof(double) * 4 * ((size_t)kParsevalBlocks + 1) + sizeof(int) * kVmaxInts;
  ok = ok && cudaMalloc(&c->pv, pv_bytes) == cudaSuccess;
  if (ok) cudaMemset(c->pv, 0, pv_bytes);
  if (ok && cfg->precision == kPrecDD)
    ok = cudaMalloc(&c->ift, sizeof(dd) * 2 * ((size_t)g.mx + g.my + g.mz)) == cudaSuccess;
  if (!ok) { free_ctx(c); g_ctx = nullptr; return fail(SAM_GPU_ECUDA, "device allocation failed"); }
  cudaMemset(c->U, 0, es * g.lu * nzmm);
  cudaMemset(c->R, 0, es * g.lu * nzmm);
  cudaMemset(c->P, 0, es * nzmm);
  DevState st{};
  st.time = 0.0;
  st.dt = cfg->dt0;
  cudaMemcpy(c->state, &st, sizeof(st), cudaMemcpyHostToDevice);
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) { free_ctx(c); g_ctx = nullptr; return fail(SAM_GPU_ECUDA, "init: %s", cudaGetErrorString(e)); }
  return 0;
}

int sam_gpu_finalize(void) {
  if (g_ens) {
    ensemble_free();
    return 0;
  }
  if (g_ctx) { cudaStreamSynchronize(g_ctx->stream); free_ctx(g_ctx); g_ctx = nullptr; }
  return 0;
}

// ------------------------------------------------------------------ ensemble
static void ensemble_free() {
  if (!g_ens) return;
  for (Ctx* m : g_ens->members) {
    cudaStreamSynchronize(m->stream);
    free_ctx(m);
  }
  if (g_ens->gexec) cudaGraphExecDestroy(g_ens->gexec);
  for (auto& s : g_ens->stages) ens_free_stage(s);
  cudaFree(g_ens->err);
  for (cudaEvent_t e : g_ens->events) cudaEventDestroy(e);
  if (g_ens->stream) cudaStreamDestroy(g_ens->stream);
  delete g_ens;
  g_ens = nullptr;
  g_ctx = nullptr;
}

int sam_gpu_ensemble_create(const sam_gpu_config* cfgs, int n) {
  if (!cfgs || n < 1) return fail(SAM_GPU_EINVAL, "ensemble_create: need at least one configuration");
  if (g_ens) ensemble_free();
  if (g_ctx) { free_ctx(g_ctx); g_ctx = nullptr; }
  g_ens = new Ensemble();
  for (int m = 0; m < n; ++m) {
    g_ctx = nullptr;
    const int rc = init_ctx(&cfgs[m]);
    if (rc) {
      ensemble_free();
      return rc;
    }
    g_ens->members.push_back(g_ctx);
  }
  g_ctx = g_ens->members[0];
  CK(cudaStreamCreateWithFlags(&g_ens->stream, cudaStreamNonBlocking));
  g_ens->events.resize((size_t)n + 1);
  for (auto& e : g_ens->events) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  CK(cudaMalloc(&g_ens->err, sizeof(int)));
  CK(cudaMemset(g_ens->err, 0, sizeof(int)));
  return 0;
}

int sam_gpu_ensemble_set_persistent(int ctas_per_sm) {
  if (!g_ens) return fail(SAM_GPU_ENOTINIT, "no ensemble (sam_gpu_ensemble_create)");
  if (ctas_per_sm < 0 || ctas_per_sm > 3) return fail(SAM_GPU_EINVAL, "ensemble_set_persistent: 0 .. 3");
  g_ens->persistent = ctas_per_sm;
  if (g_ens->gexec) { cudaGraphExecDestroy(g_ens->gexec); g_ens->gexec = nullptr; }
  return 0;
}

int sam_gpu_ensemble_persistent_members(int* n) {
  if (!g_ens) return fail(SAM_GPU_ENOTINIT, "no ensemble (sam_gpu_ensemble_create)");
  if (!n) return fail(SAM_GPU_EINVAL, "ensemble_persistent_members: null output");
  *n = g_ens->n_persistent;
  return 0;
}

int sam_gpu_ensemble_select(int m) {
  if (!g_ens) return fail(SAM_GPU_ENOTINIT, "no ensemble (sam_gpu_ensemble_create)");
  if (m < 0 || m >= (int)g_ens->members.size()) return fail(SAM_GPU_EINVAL, "ensemble member %d out of range", m);
  g_ctx = g_ens->members[(size_t)m];
  return 0;
}

// Members the persistent stage launch takes: the FP32 bulk form without a
// subgrid closure, every transform length with a compile-time FFT path of the
// launch (32, 64, 96, 128), and tiles whose shared memory lets two CTAs share
// an SM.
static bool ens_eligible(const Ctx& c) {
  return c.cfg.precision == 32 && c.les_model == 0 && ens_length_ok(c.g.nx) && ens_length_ok(c.g.ny) &&
         ens_length_ok(c.g.nz);
}

static int enqueue_step(Ctx& c) {
  int rc = 0;
  for (int nrk = 1; nrk <= c.cfg.nrk_max && !rc; ++nrk) rc = stage_any(c, nrk);
  if (!rc && c.ou) {
    if (c.cfg.precision == 32) ou_apply<float>((float2*)c.U, c.g, c.ou, c.state, c.stream);
    else ou_apply<double>((double2*)c.U, c.g, c.ou, c.state, c.stream);
  }
  return rc;
}

int sam_gpu_ensemble_step(int nsteps) {
  if (!g_ens) return fail(SAM_GPU_ENOTINIT, "no ensemble (sam_gpu_ensemble_create)");
  if (nsteps < 0) return fail(SAM_GPU_EINVAL, "negative step count");
  Ensemble& E = *g_ens;
  // a member's settings (closure, forcing) may have changed since the graph
  // was captured: rebuild it whenever any member's own graph was dropped
  bool stale = !E.gexec;
  for (Ctx* m : E.members) stale = stale || m->graph_stale;
  if (stale) {
    if (E.gexec) { cudaGraphExecDestroy(E.gexec); E.gexec = nullptr; }
    for (Ctx* m : E.members) CK(cudaStreamSynchronize(m->stream));
    // the persistent members (larger first, so that their tiles start early
    // in each pass level) and their recorded stages
    std::vector<size_t> pm;
    std::vector<char> in_pm(E.members.size(), 0);
    if (E.persistent)
      for (size_t i = 0; i < E.members.size(); ++i)
        if (ens_eligible(*E.members[i])) pm.push_back(i);
    std::stable_sort(pm.begin(), pm.end(), [&](size_t a, size_t b) {
      const Grid &ga = E.members[a]->g, &gb = E.members[b]->g;
      return (long long)ga.nx * ga.ny * ga.nz > (long long)gb.nx * gb.ny * gb.nz;
    });
    E.recs.assign(pm.size() * 3, EnsRecorder());
    for (int s = 0; s < 3; ++s) {
      std::vector<EnsRecorder*> rs;
      for (size_t k = 0; k < pm.size(); ++k) {
        Ctx& m = *E.members[pm[k]];
        if (s + 1 > m.cfg.nrk_max) continue;
        EnsRecorder* r = &E.recs[k * 3 + (size_t)s];
        m.rec = r;
        const int rc = stage_any(m, s + 1);
        m.rec = nullptr;
        if (rc) return rc;
        rs.push_back(r);
      }
      const int brc = ens_build_stage(rs, E.stages[s]);
      if (brc == -2) return fail(SAM_GPU_EUNSUPPORTED, "ensemble stage: a member's tiles do not fit the persistent launch");
      if (brc) return fail(SAM_GPU_ECUDA, "ensemble stage: device allocation failed");
    }
    for (size_t k : pm) in_pm[k] = 1;
    E.n_persistent = (int)pm.size();
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(E.stream, cudaStreamCaptureModeThreadLocal));
    CK(cudaEventRecord(E.events.back(), E.stream));
    int rc = 0;
    for (size_t i = 0; i < E.members.size() && !rc; ++i) {
      if (in_pm[i]) continue;
      Ctx& m = *E.members[i];
      cudaStreamWaitEvent(m.stream, E.events.back(), 0);
      rc = enqueue_step(m);
      cudaEventRecord(E.events[i], m.stream);
      cudaStreamWaitEvent(E.stream, E.events[i], 0);
    }
    // the persistent members: one launch per stage on the ensemble's stream
    // (concurrent with the other members' branches), then their forcing
    if (!rc && !pm.empty()) {
      for (int s = 0; s < 3; ++s) ens_launch_stage(E.stages[s], E.persistent, E.err, E.stream);
      for (size_t k : pm) {
        Ctx& m = *E.members[k];
        if (m.ou) ou_apply<float>((float2*)m.U, m.g, m.ou, m.state, E.stream);
      }
    }
    cudaError_t e = cudaStreamEndCapture(E.stream, &graph);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(SAM_GPU_ECUDA, "ensemble graph capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&E.gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(SAM_GPU_ECUDA, "ensemble graph instantiate: %s", cudaGetErrorString(e));
    for (Ctx* m : E.members) m->graph_stale = 0;
  }
  for (int s = 0; s < nsteps; ++s) CK(cudaGraphLaunch(E.gexec, E.stream));
  for (Ctx* m : E.members) m->nrk = m->cfg.nrk_max;
  CK(cudaStreamSynchronize(E.stream));
  int herr = 0;
  CK(cudaMemcpy(&herr, E.err, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) {
    cudaMemset(E.err, 0, sizeof(int));
    return fail(SAM_GPU_ECUDA, "ensemble stage: a dependency wait of the persistent launch timed out");
  }
  return check_launch();
}

int sam_gpu_ensemble_destroy(void) {
  ensemble_free();
  return 0;
}

int sam_gpu_dims(int* o) {
  NEED_CTX();
  const Grid& g = c.g;
  o[0] = g.mx; o[1] = g.my; o[2] = g.mz; o[3] = g.nze; o[4] = g.lu; o[5] = g.lr;
  o[6] = g.kx; o[7] = g.ky; o[8] = g.kz; o[9] = c.lm; o[10] = c.nx2;
  return 0;
}

int sam_gpu_set_stream(void* s) {
  NEED_CTX();
  c.stream = s ? (cudaStream_t)s : c.own;
  c.graph_stale = 1;
  return 0;
}

int sam_gpu_set_tstep(int nrk, double dt, double time) {
  NEED_CTX();
  if (nrk < 1 || nrk > c.cfg.nrk_max) return fail(SAM_GPU_EINVAL, "nrk %d out of range", nrk);
  c.nrk = nrk;
  DevState st;
  CK(cudaMemcpyAsync(&st, c.state, sizeof(st), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  st.dt = dt;
  st.time = time;
  CK(cudaMemcpyAsync(c.state, &st, sizeof(st), cudaMemcpyHostToDevice, c.stream));
  return sync_stream(c);
}

int sam_gpu_get_stats(sam_gpu_stats* out) {
  NEED_CTX();
  DevState st;
  CK(cudaMemcpyAsync(&st, c.state, sizeof(st), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  out->time = st.time;
  out->dt = st.dt;
  for (int n = 0; n < 4; ++n) { out->u_avg[n] = st.u_avg[n]; out->u_var[n] = st.u_var[n]; out->u_max[n] = st.u_max[n]; }
  out->energy = st.energy;
  out->cfl_x = st.cfl_x; out->cfl_y = st.cfl_y; out->cfl_z = st.cfl_z;
  out->nonfinite = st.nonfinite;
  return 0;
}

// ------------------------------------------------------ per-routine drop-ins

static bool symm_ok(const int* isymm, int n_var) {
  if (!isymm) return true;
  for (int n = 0; n < n_var; ++n)
    if (isymm[n] != 0) return false;
  return true;
}

int sam_gpu_z_trans_b(const double* u1, double* u2, int n_var, const int* isymm, double*, double*, double*) {
  NEED_CTX();
  const Grid& g = c.g;
  if (n_var < 1 || !u1 || !u2) return fail(SAM_GPU_EINVAL, "z_trans_b: bad arguments");
  if (!symm_ok(isymm, n_var)) return fail(SAM_GPU_EUNSUPPORTED, "z_trans_b: only the periodic branch (isymm=0) exists");
  const size_t nin = (size_t)g.nze * g.my * g.mx * n_var, nout = (size_t)g.my * g.mx * g.nze * n_var;
  int rc;
  if ((rc = ensure(c.sc[0], nin * 16)) || (rc = ensure(c.sc[1], nout * 16))) return rc;
  CK(cudaMemcpyAsync(c.sc[0].p, u1, nin * 16, cudaMemcpyHostToDevice, c.stream));
  rc = run_z_inv<double>(c, c.sc[0].p, c.sc[1].p, n_var, g.nze, (long long)g.my * g.nze,
                         (long long)g.mx * g.my * g.nze, g.my, (long long)g.mx * g.my, (long long)g.nze * g.mx * g.my);
  if (rc) return rc;
  CK(cudaMemcpyAsync(u2, c.sc[1].p, nout * 16, cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

int sam_gpu_x2z_decomp(double* u1, double* u2, int n_var, double*) {
  NEED_CTX();
  const Grid& g = c.g;
  if (n_var < 1 || !u1 || !u2) return fail(SAM_GPU_EINVAL, "x2z_decomp: bad arguments");
  const size_t nin = (size_t)g.my * g.mx * g.nze * n_var;
  const size_t nout = (size_t)g.ny * c.nx2 * g.nz * n_var;
  int rc;
  if ((rc = ensure(c.sc[0], nin * 16)) || (rc = ensure(c.sc[1], nout * 16))) return rc;
  CK(cudaMemcpyAsync(c.sc[0].p, u1, nin * 16, cudaMemcpyHostToDevice, c.stream));
  launch_x2z((const double2*)c.sc[0].p, (double2*)c.sc[1].p, g, n_var, c.nx2, c.stream);
  // only the columns kx < Nx_min of each (z, var) plane are written back
  CK(cudaMemcpy2DAsync(u2, (size_t)g.ny * c.nx2 * 16, c.sc[1].p, (size_t)g.ny * c.nx2 * 16, (size_t)g.ny * g.mx * 16,
                       (size_t)g.nz * n_var, cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

int sam_gpu_xy_trans_b(double* u1, double* u2, int n_var, double*) {
  NEED_CTX();
  const Grid& g = c.g;
  if (n_var < 1 || !u1 || !u2) return fail(SAM_GPU_EINVAL, "xy_trans_b: bad arguments");
  const size_t nin = (size_t)g.ny * c.nx2 * g.nz * n_var;  // complex
  const size_t nb = (size_t)n_var * g.nz * g.ny * g.mx;    // complex
  const size_t nout = (size_t)g.nx * g.ny * g.nz * n_var;  // real
  int rc;
  if ((rc = ensure(c.sc[0], nin * 16)) || (rc = ensure(c.sc[1], nb * 16)) || (rc = ensure(c.sc[2], nout * 8)))
    return rc;
  CK(cudaMemcpyAsync(c.sc[0].p, u1, nin * 16, cudaMemcpyHostToDevice, c.stream));
  rc = run_y_inv<double>(c, c.sc[0].p, c.sc[1].p, n_var, 1, g.ny, (long long)g.ny * c.nx2,
                         (long long)g.ny * c.nx2 * g.nz, g.mx, (long long)g.ny * g.mx, (long long)g.nz * g.ny * g.mx);
  if (rc) return rc;
  rc = run_x_pass<double>(c, 0, 0, n_var, c.sc[1].p, nullptr, g.mx, (long long)g.ny * g.mx,
                          (long long)g.nz * g.ny * g.mx, nullptr, c.sc[2].p, 0, 0, 0, g.nx, (long long)g.nx * g.ny,
                          (long long)g.nx * g.ny * g.nz, false);
  if (rc) return rc;
  CK(cudaMemcpyAsync(u2, c.sc[2].p, nout * 8, cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

int sam_gpu_xy_trans_f(double* u1, double* u2, int n_var, double*) {
  NEED_CTX();
  const Grid& g = c.g;
  if (n_var < 1 || !u1 || !u2) return fail(SAM_GPU_EINVAL, "xy_trans_f: bad arguments");
  const size_t nin = (size_t)g.nx * g.ny * g.nz * n_var;   // real
  const size_t nc = (size_t)n_var * g.nz * g.mx * g.ny;    // complex
  const size_t nout = (size_t)g.nze * g.my * g.mx * n_var; // complex
  int rc;
  if ((rc = ensure(c.sc[0], nin * 8)) || (rc = ensure(c.sc[1], nc * 16)) || (rc = ensure(c.sc[2], nout * 16)))
    return rc;
  CK(cudaMemcpyAsync(c.sc[0].p, u1, nin * 8, cudaMemcpyHostToDevice, c.stream));
  rc = run_x_pass<double>(c, 1, 1, n_var, nullptr, c.sc[0].p, g.nx, (long long)g.nx * g.ny,
                          (long long)g.nx * g.ny * g.nz, c.sc[1].p, nullptr, g.ny, (long long)g.mx * g.ny,
                          (long long)g.nz * g.mx * g.ny, 0, 0, 0, false);
  if (rc) return rc;
  rc = run_y_fwd<double>(c, c.sc[1].p, c.sc[2].p, n_var, g.ny, (long long)g.mx * g.ny, (long long)g.nz * g.mx * g.ny,
                         g.nze, (long long)g.my * g.nze, (long long)g.mx * g.my * g.nze);
  if (rc) return rc;
  CK(cudaMemcpyAsync(u2, c.sc[2].p, nout * 16, cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

int sam_gpu_z2x_decomp(double* u1, double* u2, int n_var, double*) {
  NEED_CTX();
  const Grid& g = c.g;
  if (n_var < 1 || !u1 || !u2) return fail(SAM_GPU_EINVAL, "z2x_decomp: bad arguments");
  // one rank: the received blocks (nzp, Ny_min, nxp, n_var) are the output layout
  if (u1 != u2) memmove(u2, u1, (size_t)g.nze * g.my * g.mx * n_var * 16);
  return 0;
}

int sam_gpu_z_trans_f(double* u, int n_var, const int* isymm, double*, double*) {
  NEED_CTX();
  const Grid& g = c.g;
  if (n_var < 1 || !u) return fail(SAM_GPU_EINVAL, "z_trans_f: bad arguments");
  if (!symm_ok(isymm, n_var)) return fail(SAM_GPU_EUNSUPPORTED, "z_trans_f: only the periodic branch (isymm=0) is supported");
  const size_t n = (size_t)g.nze * g.my * g.mx * n_var;
  int rc;
  if ((rc = ensure(c.sc[0], n * 16))) return rc;
  CK(cudaMemcpyAsync(c.sc[0].p, u, n * 16, cudaMemcpyHostToDevice, c.stream));
  ZFwdArgs<double> a{};
  a.in = (double2*)c.sc[0].p;
  a.mode = 0;
  a.nf = n_var;
  a.in_ky = g.nze; a.in_kx = (long long)g.my * g.nze; a.in_n = (long long)g.mx * g.my * g.nze;
  if ((rc = run_z_fwd<double>(c, a))) return rc;
  CK(cudaMemcpyAsync(u, c.sc[0].p, n * 16, cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

int sam_gpu_vel_max(const double* u, double*) {
  NEED_CTX();
  const Grid& g = c.g;
  if (!u) return fail(SAM_GPU_EINVAL, "vel_max: null array");
  const size_t n = (size_t)g.nx * g.ny * g.nz * g.lu;
  int rc;
  if ((rc = ensure(c.sc[0], n * 8))) return rc;
  CK(cudaMemcpyAsync(c.sc[0].p, u, n * 8, cudaMemcpyHostToDevice, c.stream));
  rc = run_x_pass<double>(c, 1, 3, g.lu, nullptr, c.sc[0].p, g.nx, (long long)g.nx * g.ny,
                          (long long)g.nx * g.ny * g.nz, nullptr, nullptr, 0, 0, 0, 0, 0, 0, true);
  if (rc) return rc;
  return sync_stream(c);
}

int sam_gpu_rhs(double* u, double* uu, double* r, const double* u_sav, double*) {
  NEED_CTX();
  const Grid& g = c.g;
  if (!uu || !r) return fail(SAM_GPU_EINVAL, "rhs: null array");
  if (c.cfg.i_strat && !u_sav) return fail(SAM_GPU_EINVAL, "rhs: u_sav is required when stratified");
  (void)u;  // u and uu are the same array in sam.f:244; the physical fields are read from uu
  const size_t nphys = (size_t)g.nx * g.ny * g.nz * g.lu;
  const size_t nc = (size_t)g.lr * g.nz * g.mx * g.ny;
  const size_t nd = (size_t)g.lr * g.mx * g.my * g.nze;
  const size_t nr = (size_t)(g.lu + 1) * g.mx * g.my * g.nze;
  const size_t ns = (size_t)2 * g.mz * g.my * g.mx;
  int rc;
  if ((rc = ensure(c.sc[0], nphys * 8)) || (rc = ensure(c.sc[1], nc * 16)) || (rc = ensure(c.sc[2], nd * 16)) ||
      (rc = ensure(c.sc[3], (nr + ns) * 16)))
    return rc;
  CK(cudaMemcpyAsync(c.sc[0].p, uu, nphys * 8, cudaMemcpyHostToDevice, c.stream));
  double2* dr = (double2*)c.sc[3].p;
  double2* dsav = dr + nr;
  if (c.cfg.i_strat) CK(cudaMemcpyAsync(dsav, u_sav, ns * 16, cudaMemcpyHostToDevice, c.stream));
  rc = run_x_pass<double>(c, 1, 2, g.lu, nullptr, c.sc[0].p, g.nx, (long long)g.nx * g.ny,
                          (long long)g.nx * g.ny * g.nz, c.sc[1].p, nullptr, g.ny, (long long)g.mx * g.ny,
                          (long long)g.nz * g.mx * g.ny, 0, 0, 0, c.nrk == 1);
  if (rc) return rc;
  rc = run_y_fwd<double>(c, c.sc[1].p, c.sc[2].p, g.lr, g.ny, (long long)g.mx * g.ny, (long long)g.nz * g.mx * g.ny,
                         g.nze, (long long)g.my * g.nze, (long long)g.mx * g.my * g.nze);
  if (rc) return rc;
  ZFwdArgs<double> a{};
  a.in = (double2*)c.sc[2].p;
  a.mode = 1;
  a.nf = g.lr;
  a.in_ky = g.nze; a.in_kx = (long long)g.my * g.nze; a.in_n = (long long)g.mx * g.my * g.nze;
  a.r = dr;
  a.r_ky = g.nze; a.r_kx = (long long)g.my * g.nze; a.r_n = (long long)g.mx * g.my * g.nze;
  a.usav = dsav;
  a.sav_ky = g.mz; a.sav_kx = (long long)g.my * g.mz; a.sav_n = (long long)g.mx * g.my * g.mz;
  a.state = c.state;
  a.sc = stage_consts(c, c.nrk, 1);
  if ((rc = run_z_fwd<double>(c, a))) return rc;
  // rows 1..Nz_min of r(:,:,:,1..Lu+1)
  CK(cudaMemcpy2DAsync(r, (size_t)g.nze * 16, dr, (size_t)g.nze * 16, (size_t)g.mz * 16,
                       (size_t)g.my * g.mx * (g.lu + 1), cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

// ------------------------------------------------------------ resident path

int sam_gpu_upload(const double* u) {
  NEED_CTX();
  const Grid& g = c.g;
  if (!u) return fail(SAM_GPU_EINVAL, "upload: null array");
  const size_t nm = (size_t)g.mx * g.my * g.mz * g.lu;
  int rc;
  void* dst = c.U;
  if (c.cfg.precision != 64) {
    if ((rc = ensure(c.sc[0], nm * 16))) return rc;
    dst = c.sc[0].p;
  }
  // rows 1..Nz_min of each (ky, kx, var) column of u(Nze,Ny_min,nxp,Lu)
  CK(cudaMemcpy2DAsync(dst, (size_t)g.mz * 16, u, (size_t)g.nze * 16, (size_t)g.mz * 16, (size_t)g.my * g.mx * g.lu,
                       cudaMemcpyHostToDevice, c.stream));
  if (c.cfg.precision != 64) state_from_fp64(c, (const double2*)dst, c.U, (long long)nm);
  CK(cudaMemsetAsync(c.R, 0, csize(c) * nm, c.stream));
  return sync_stream(c);
}

static int download_field(Ctx& c, const void* src, double* host, int nf, int host_field0) {
  const Grid& g = c.g;
  const size_t nm = (size_t)g.mx * g.my * g.mz * nf;
  const void* s = src;
  int rc;
  if (c.cfg.precision != 64) {
    if ((rc = ensure(c.sc[1], nm * 16))) return rc;
    state_to_fp64(c, src, (double2*)c.sc[1].p, (long long)nm);
    s = c.sc[1].p;
  }
  double* h = host + (size_t)2 * g.nze * g.my * g.mx * host_field0;
  CK(cudaMemcpy2DAsync(h, (size_t)g.nze * 16, s, (size_t)g.mz * 16, (size_t)g.mz * 16, (size_t)g.my * g.mx * nf,
                       cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

int sam_gpu_download(double* u, double* r) {
  NEED_CTX();
  int rc;
  if (u && (rc = download_field(c, c.U, u, c.g.lu, 0))) return rc;
  if (r) {
    if ((rc = download_field(c, c.R, r, c.g.lu, 0))) return rc;
    if ((rc = download_field(c, c.P, r, 1, c.g.lu))) return rc;
  }
  return 0;
}

int sam_gpu_stage(int nrk) {
  NEED_CTX();
  if (nrk < 1 || nrk > c.cfg.nrk_max) return fail(SAM_GPU_EINVAL, "nrk %d out of range", nrk);
  int rc = stage_any(c, nrk);
  if (rc) return rc;
  c.nrk = nrk;
  return check_launch();
}

int sam_gpu_step(int nsteps) {
  NEED_CTX();
  if (nsteps < 0) return fail(SAM_GPU_EINVAL, "negative step count");
  if (!c.gexec || c.graph_stream != c.stream) {
    if (c.gexec) { cudaGraphExecDestroy(c.gexec); c.gexec = nullptr; }
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    for (int nrk = 1; nrk <= c.cfg.nrk_max && !rc; ++nrk) rc = stage_any(c, nrk);
    if (!rc && c.ou) {
      if (c.cfg.precision == 32) ou_apply<float>((float2*)c.U, c.g, c.ou, c.state, c.stream);
      else ou_apply<double>((double2*)c.U, c.g, c.ou, c.state, c.stream);
    }
    cudaError_t e = cudaStreamEndCapture(c.stream, &graph);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(SAM_GPU_ECUDA, "graph capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&c.gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(SAM_GPU_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
    c.graph_stream = c.stream;
  }
  for (int s = 0; s < nsteps; ++s) CK(cudaGraphLaunch(c.gexec, c.stream));
  c.nrk = c.cfg.nrk_max;
  return check_launch();
}

int sam_gpu_set_forcing(unsigned long long seed, double k_f, double sigma, double t_l, int* n_modes) {
  NEED_CTX();
  if (n_modes) *n_modes = 0;
  if (c.cfg.precision == kPrecDD && k_f > 0.0 && sigma != 0.0)
    return fail(SAM_GPU_EUNSUPPORTED, "set_forcing: the double-float form runs the plain step only");
  if (c.gexec) { cudaGraphExecDestroy(c.gexec); c.gexec = nullptr; }
  c.graph_stale = 1;
  if (k_f <= 0.0 || sigma == 0.0) {
    cudaFree(c.ou);
    c.ou = nullptr;
    return 0;
  }
  if (!(t_l > 0.0) || !(sigma > 0.0) || !(k_f < 1e3))
    return fail(SAM_GPU_EINVAL, "set_forcing: need sigma > 0, T_L > 0 and a finite k_f");
  OuForcing h{};
  const int n = ou_modes(c.g, k_f, h);
  if (n < 0) return fail(SAM_GPU_EINVAL, "set_forcing: more than %d modes with |k| <= %g", kOuModesMax, k_f);
  if (n == 0) return fail(SAM_GPU_EINVAL, "set_forcing: no stored mode with 0 < |k| <= %g", k_f);
  h.seed = seed;
  h.sigma = sigma;
  h.t_l = t_l;
  if (!c.ou) CK(cudaMalloc(&c.ou, sizeof(OuForcing)));
  CK(cudaMemcpyAsync(c.ou, &h, sizeof(OuForcing), cudaMemcpyHostToDevice, c.stream));
  ou_init(c.ou, c.stream);
  if (n_modes) *n_modes = n;
  return sync_stream(c);
}

static int mlp_ensure(Ctx& c);

int sam_gpu_set_les(int model, double c_smag, double pr_t) {
  NEED_CTX();
  if (model != 0 && c.cfg.precision == kPrecDD)
    return fail(SAM_GPU_EUNSUPPORTED, "set_les: the double-float form runs the plain step only");
  if (model < 0 || model > 3)
    return fail(SAM_GPU_EINVAL, "set_les: model %d (0 off, 1 Smagorinsky, 2 dynamic, 3 learned)", model);
  if (!(pr_t > 0.0)) return fail(SAM_GPU_EINVAL, "set_les: turbulent Prandtl number must be > 0");
  if (model == 1 && !(c_smag >= 0.0)) return fail(SAM_GPU_EINVAL, "set_les: c_smag must be >= 0");
  if (c.gexec) { cudaGraphExecDestroy(c.gexec); c.gexec = nullptr; }
  c.graph_stale = 1;
  CK(cudaStreamSynchronize(c.stream));
  const Grid& g = c.g;
  const size_t es = csize(c);
  if (model) {
    // pencil buffers for the Lr gradient fields beside the Lu fields
    const int nf = g.lu + g.lr + (model == 3 ? 3 : 0);
    const size_t s1 = (size_t)nf * g.mx * g.my * g.nz;
    const size_t s2 = (size_t)nf * g.nz * g.ny * g.mx;
    if (c.s1_elems < s1) {
      cudaFree(c.S1); c.S1 = nullptr; c.s1_elems = 0;
      CK(cudaMalloc(&c.S1, es * s1));
      c.s1_elems = s1;
    }
    if (c.s2_elems < s2) {
      cudaFree(c.S2); c.S2 = nullptr; c.s2_elems = 0;
      CK(cudaMalloc(&c.S2, es * s2));
      c.s2_elems = s2;
    }
    if (!c.les_cds) CK(cudaMalloc(&c.les_cds, sizeof(double)));
    if (model == 2 && !c.les_work) {
      CK(cudaMalloc(&c.les_phys, (es / 2) * 3 * (size_t)g.nx * g.ny * g.nz));
      CK(cudaMalloc(&c.les_work, sizeof(double) * les_dynamic_work(g.nx, g.ny, g.nz)));
    }
    if (model == 3 && !c.les_feat) {
      const size_t np = (size_t)g.nx * g.ny * g.nz;
      int rc = mlp_ensure(c);
      if (rc) return rc;
      CK(cudaMalloc(&c.les_feat, 32 * np));
      CK(cudaMalloc(&c.les_coef, sizeof(float2) * np));
      // zero until the first stage 1 forms them (no subgrid terms before)
      CK(cudaMemsetAsync(c.les_coef, 0, sizeof(float2) * np, c.stream));
    }
  }
  double dsq;
  grid_spacing(c, c.les_dxi, c.les_dyi, c.les_dzi, dsq);
  c.les_dsq = dsq;
  c.les_model = model;
  c.les_prt_inv = 1.0 / pr_t;
  if (model) {
    // sm.f:32 (model 1); the dynamic coefficient starts at 0 and is set at
    // stage 1 of every step (model 2)
    const double cds = model == 1 ? c_smag * dsq : 0.0;
    CK(cudaMemcpy(c.les_cds, &cds, sizeof(double), cudaMemcpyHostToDevice));
  }
  return 0;
}

int sam_gpu_les_coef(double* c_delta_sq) {
  NEED_CTX();
  if (!c_delta_sq) return fail(SAM_GPU_EINVAL, "les_coef: null output");
  *c_delta_sq = 0.0;
  if (!c.les_model) return 0;
  CK(cudaMemcpyAsync(c_delta_sq, c.les_cds, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

// ---------------------------------------------------------- learned closure
static int mlp_ensure(Ctx& c) {
  if (c.mlp_p) return 0;
  CK(cudaMalloc(&c.mlp_p, sizeof(float) * kMlpParams));
  CK(cudaMalloc(&c.mlp_m, sizeof(float) * kMlpParams));
  CK(cudaMalloc(&c.mlp_v, sizeof(float) * kMlpParams));
  CK(cudaMalloc(&c.mlp_g, sizeof(float) * kMlpParams));
  CK(cudaMalloc(&c.mlp_loss, sizeof(float) * 4));
  CK(cudaMalloc(&c.mlp_dev, sizeof(MlpDev)));
  CK(cudaMalloc(&c.mlp_err, sizeof(int)));
  CK(cudaMemset(c.mlp_p, 0, sizeof(float) * kMlpParams));
  CK(cudaMemset(c.mlp_m, 0, sizeof(float) * kMlpParams));
  CK(cudaMemset(c.mlp_v, 0, sizeof(float) * kMlpParams));
  CK(cudaMemset(c.mlp_err, 0, sizeof(int)));
  mlp_pack(c.mlp_p, c.mlp_dev, c.stream);
  return 0;
}

static int mlp_check_err(Ctx& c) {
  int e = 0;
  CK(cudaMemcpyAsync(&e, c.mlp_err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (e) {
    cudaMemsetAsync(c.mlp_err, 0, sizeof(int), c.stream);
    return fail(SAM_GPU_ECUDA, "closure network: tensor-core wait timed out");
  }
  return check_launch();
}

int sam_gpu_mlp_set(const float* params, int n) {
  NEED_CTX();
  if (!params || n != kMlpParams) return fail(SAM_GPU_EINVAL, "mlp_set: need %d parameters", kMlpParams);
  int rc = mlp_ensure(c);
  if (rc) return rc;
  CK(cudaMemcpyAsync(c.mlp_p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, c.stream));
  CK(cudaMemsetAsync(c.mlp_m, 0, sizeof(float) * kMlpParams, c.stream));
  CK(cudaMemsetAsync(c.mlp_v, 0, sizeof(float) * kMlpParams, c.stream));
  c.mlp_step = 0;
  mlp_pack(c.mlp_p, c.mlp_dev, c.stream);
  return sync_stream(c);
}

int sam_gpu_mlp_get(float* params, int n) {
  NEED_CTX();
  if (!params || n != kMlpParams) return fail(SAM_GPU_EINVAL, "mlp_get: need %d parameters", kMlpParams);
  int rc = mlp_ensure(c);
  if (rc) return rc;
  CK(cudaMemcpyAsync(params, c.mlp_p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

// features [n][12] (host, FP32) into sc[0] as BF16 [n][16]; sc[1] gets
// room for `extra` more bytes after the coefficients
static int mlp_stage_inputs(Ctx& c, const float* feat, long long n, __nv_bfloat16** x16) {
  int rc;
  const size_t fb = sizeof(float) * kMlpIn * (size_t)n;
  if ((rc = ensure(c.sc[2], fb)) || (rc = ensure(c.sc[0], sizeof(__nv_bfloat16) * kMlpK1 * (size_t)n))) return rc;
  CK(cudaMemcpyAsync(c.sc[2].p, feat, fb, cudaMemcpyHostToDevice, c.stream));
  mlp_features_bf16((const float*)c.sc[2].p, (__nv_bfloat16*)c.sc[0].p, n, c.stream);
  *x16 = (__nv_bfloat16*)c.sc[0].p;
  return 0;
}

int sam_gpu_mlp_forward(const float* feat, long long n, float* coef) {
  NEED_CTX();
  if (!feat || !coef || n < 0) return fail(SAM_GPU_EINVAL, "mlp_forward: bad arguments");
  if (n == 0) return 0;
  int rc = mlp_ensure(c);
  if (rc) return rc;
  __nv_bfloat16* x16;
  if ((rc = mlp_stage_inputs(c, feat, n, &x16)) || (rc = ensure(c.sc[1], sizeof(float2) * (size_t)n))) return rc;
  if (mlp_forward(x16, n, c.mlp_dev, (float2*)c.sc[1].p, nullptr, c.mlp_err, c.stream) < 0)
    return fail(SAM_GPU_ECUDA, "closure network: no TMA tensor map");
  CK(cudaMemcpyAsync(coef, c.sc[1].p, sizeof(float2) * (size_t)n, cudaMemcpyDeviceToHost, c.stream));
  return mlp_check_err(c);
}

// device buffers of one minibatch of up to nb points: targets, activations,
// outputs and gradient partials, carved from sc[3]
struct MlpWork {
  float2* y;
  float2* coef;
  MlpBatch b;
  float* part;
};
static int mlp_work(Ctx& c, long long nb, MlpWork& w) {
  const size_t need = sizeof(float2) * nb * 2 + sizeof(__nv_bfloat16) * kMlpH * nb * 2 + sizeof(float) * 2 * nb +
                      sizeof(float) * (size_t)mlp_partials(nb) + 256 * 6;
  int rc = ensure(c.sc[3], need);
  if (rc) return rc;
  uint8_t* p = (uint8_t*)c.sc[3].p;
  auto take = [&](size_t bytes) {
    uint8_t* q = p;
    p += (bytes + 255) & ~(size_t)255;
    return q;
  };
  w.y = (float2*)take(sizeof(float2) * nb);
  w.coef = (float2*)take(sizeof(float2) * nb);
  w.b.h1 = (__nv_bfloat16*)take(sizeof(__nv_bfloat16) * kMlpH * nb);
  w.b.h2 = (__nv_bfloat16*)take(sizeof(__nv_bfloat16) * kMlpH * nb);
  w.b.o = (float*)take(sizeof(float) * 2 * nb);
  w.part = (float*)take(sizeof(float) * (size_t)mlp_partials(nb));
  return 0;
}

int sam_gpu_mlp_grad(const float* feat, const float* target, long long n, float* grad, float* loss) {
  NEED_CTX();
  if (!feat || !target || !grad || n <= 0) return fail(SAM_GPU_EINVAL, "mlp_grad: bad arguments");
  int rc = mlp_ensure(c);
  if (rc) return rc;
  __nv_bfloat16* x16;
  MlpWork w;
  if ((rc = mlp_stage_inputs(c, feat, n, &x16)) || (rc = mlp_work(c, n, w))) return rc;
  CK(cudaMemcpyAsync(w.y, target, sizeof(float2) * (size_t)n, cudaMemcpyHostToDevice, c.stream));
  if (mlp_forward(x16, n, c.mlp_dev, w.coef, &w.b, c.mlp_err, c.stream) < 0)
    return fail(SAM_GPU_ECUDA, "closure network: no TMA tensor map");
  mlp_backward(x16, w.y, n, c.mlp_dev, w.b, w.part, c.mlp_g, c.mlp_loss, c.mlp_err, c.mlp_tc_bwd != 0, c.stream);
  CK(cudaMemcpyAsync(grad, c.mlp_g, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, c.stream));
  float ls = 0.f;
  CK(cudaMemcpyAsync(&ls, c.mlp_loss, sizeof(float), cudaMemcpyDeviceToHost, c.stream));
  rc = mlp_check_err(c);
  if (loss) *loss = ls / (2.0f * (float)n);
  return rc;
}

int sam_gpu_mlp_set_backward(int tensor_cores) {
  NEED_CTX();
  if (tensor_cores != 0 && tensor_cores != 1) return fail(SAM_GPU_EINVAL, "mlp_set_backward: 0 or 1");
  c.mlp_tc_bwd = tensor_cores;
  return 0;
}

int sam_gpu_mlp_train(const float* feat, const float* target, long long n, int steps, int batch, float lr,
                      float* loss_hist) {
  NEED_CTX();
  if (!feat || !target || n <= 0 || steps < 0 || batch <= 0 || !(lr > 0.f))
    return fail(SAM_GPU_EINVAL, "mlp_train: bad arguments");
  int rc = mlp_ensure(c);
  if (rc) return rc;
  const long long nb = batch < n ? batch : n;
  __nv_bfloat16* x16;
  MlpWork w;
  if ((rc = mlp_stage_inputs(c, feat, n, &x16)) || (rc = mlp_work(c, nb, w))) return rc;
  // all targets on the device; minibatch s is the contiguous chunk s (mod the
  // number of full chunks) of the data as given (the caller shuffles)
  if ((rc = ensure(c.sc[2], sizeof(float2) * (size_t)n))) return rc;
  float2* y_all = (float2*)c.sc[2].p;
  CK(cudaMemcpyAsync(y_all, target, sizeof(float2) * (size_t)n, cudaMemcpyHostToDevice, c.stream));
  const long long nchunks = n / nb;
  std::vector<float> hist((size_t)steps);
  for (int s = 0; s < steps; ++s) {
    const long long off = (s % nchunks) * nb;
    if (mlp_forward(x16 + off * kMlpK1, nb, c.mlp_dev, w.coef, &w.b, c.mlp_err, c.stream) < 0)
      return fail(SAM_GPU_ECUDA, "closure network: no TMA tensor map");
    mlp_backward(x16 + off * kMlpK1, y_all + off, nb, c.mlp_dev, w.b, w.part, c.mlp_g, c.mlp_loss + 0, c.mlp_err,
                 c.mlp_tc_bwd != 0, c.stream);
    mlp_adam(c.mlp_p, c.mlp_m, c.mlp_v, c.mlp_g, ++c.mlp_step, lr, c.mlp_dev, c.stream);
    if (loss_hist) CK(cudaMemcpyAsync(&hist[s], c.mlp_loss, sizeof(float), cudaMemcpyDeviceToHost, c.stream));
  }
  rc = mlp_check_err(c);
  if (loss_hist)
    for (int s = 0; s < steps; ++s) loss_hist[s] = hist[s] / (2.0f * (float)nb);
  return rc;
}

}  // extern "C"

// The resident state's physical fields (Lu) into sc[0] (working precision).
template <typename T>
static int physical_fields(Ctx& c) {
  const Grid& g = c.g;
  const size_t nm = (size_t)g.mx * g.my * g.mz, vol = (size_t)g.nx * g.ny * g.nz;
  const size_t es = sizeof(cx_t<T>);
  int rc;
  if ((rc = ensure(c.sc[0], vol * g.lu * sizeof(T))) || (rc = ensure(c.sc[1], es * g.lu * g.nz * g.mx * g.my)) ||
      (rc = ensure(c.sc[2], es * g.lu * g.nz * g.ny * g.mx)))
    return rc;
  if ((rc = run_z_inv<T>(c, c.U, c.sc[1].p, g.lu, g.mz, (long long)g.my * g.mz, (long long)nm, g.my,
                         (long long)g.mx * g.my, (long long)g.nz * g.mx * g.my)))
    return rc;
  if ((rc = run_y_inv<T>(c, c.sc[1].p, c.sc[2].p, g.lu, 0, g.my, (long long)g.mx * g.my,
                         (long long)g.nz * g.mx * g.my, g.mx, (long long)g.ny * g.mx, (long long)g.nz * g.ny * g.mx)))
    return rc;
  return run_x_pass<T>(c, 0, 0, g.lu, c.sc[2].p, nullptr, g.mx, (long long)g.ny * g.mx, (long long)g.nz * g.ny * g.mx,
                       nullptr, c.sc[0].p, 0, 0, 0, g.nx, (long long)g.nx * g.ny, (long long)vol, false);
}

template <typename T>
static int box_filter_impl(Ctx& c, int f, double* out) {
  const Grid& g = c.g;
  int rc = physical_fields<T>(c);
  if (rc) return rc;
  const size_t nc = (size_t)(g.nx / f) * (g.ny / f) * (g.nz / f), nfo = (size_t)(g.lu + g.lr);
  if ((rc = ensure(c.sc[3], nc * nfo * 8))) return rc;
  les_box_filter<T>((const T*)c.sc[0].p, g.lu, g.nx, g.ny, g.nz, f, (double*)c.sc[3].p, c.stream);
  CK(cudaMemcpyAsync(out, c.sc[3].p, nc * nfo * 8, cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

extern "C" {

int sam_gpu_box_filter(int f, double* out) {
  NEED_CTX();
  const Grid& g = c.g;
  if (!out || f < 1 || g.nx % f || g.ny % f || g.nz % f)
    return fail(SAM_GPU_EINVAL, "box_filter: the grid must divide into blocks of %d", f);
  if (c.cfg.precision == kPrecDD) return fail(SAM_GPU_EUNSUPPORTED, "box_filter: not in the double-float form");
  return c.cfg.precision == 32 ? box_filter_impl<float>(c, f, out) : box_filter_impl<double>(c, f, out);
}

}  // extern "C"

template <typename T>
static int closure_inputs_impl(Ctx& c, unsigned short* feat, double* grads) {
  const Grid& g = c.g;
  const int nf = g.lu + g.lr + 3, ng = g.lr + 3;
  const size_t nm = (size_t)g.mx * g.my * g.mz, vol = (size_t)g.nx * g.ny * g.nz;
  const size_t es = sizeof(cx_t<T>);
  const long long bn = (long long)g.nz * g.ny * g.mx;
  int rc;
  if ((rc = ensure(c.sc[0], vol * ng * sizeof(T))) || (rc = ensure(c.sc[1], es * nf * g.nz * g.mx * g.my)) ||
      (rc = ensure(c.sc[2], es * nf * g.nz * g.ny * g.mx)) || (rc = ensure(c.sc[3], vol * ng * 8)))
    return rc;
  if (!c.les_feat) CK(cudaMalloc(&c.les_feat, 32 * vol));
  if ((rc = run_z_inv<T>(c, c.U, c.sc[1].p, nf, g.mz, (long long)g.my * g.mz, (long long)nm, g.my,
                         (long long)g.mx * g.my, (long long)g.nz * g.mx * g.my, 1)))
    return rc;
  if ((rc = run_y_inv<T>(c, c.sc[1].p, c.sc[2].p, nf, 0, g.my, (long long)g.mx * g.my,
                         (long long)g.nz * g.mx * g.my, g.mx, (long long)g.ny * g.mx, bn)))
    return rc;
  const cx_t<T>* gin = (const cx_t<T>*)c.sc[2].p + g.lu * bn;
  if ((rc = run_x_pass<T>(c, 0, 0, ng, gin, nullptr, g.mx, (long long)g.ny * g.mx, bn, nullptr, c.sc[0].p, 0, 0, 0,
                          g.nx, (long long)g.nx * g.ny, (long long)vol, false)))
    return rc;
  if ((rc = run_x_pass<T>(c, 0, 4, ng, gin, nullptr, g.mx, (long long)g.ny * g.mx, bn, nullptr, nullptr, 0, 0, 0, 0,
                          0, 0, false)))
    return rc;
  les_to_double<T>((const T*)c.sc[0].p, (double*)c.sc[3].p, (long long)(vol * ng), c.stream);
  if (grads) CK(cudaMemcpyAsync(grads, c.sc[3].p, vol * ng * 8, cudaMemcpyDeviceToHost, c.stream));
  if (feat) CK(cudaMemcpyAsync(feat, c.les_feat, 32 * vol, cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

extern "C" {

int sam_gpu_closure_inputs(unsigned short* feat, double* grads) {
  NEED_CTX();
  double dsq, dxi, dyi, dzi;
  grid_spacing(c, dxi, dyi, dzi, dsq);
  c.les_dsq = dsq;
  if (c.cfg.precision == kPrecDD) return fail(SAM_GPU_EUNSUPPORTED, "closure_inputs: not in the double-float form");
  return c.cfg.precision == 32 ? closure_inputs_impl<float>(c, feat, grads)
                               : closure_inputs_impl<double>(c, feat, grads);
}

int sam_gpu_mma_selftest(const float* a, const float* b, float* d) {
  NEED_CTX();
  if (!a || !b || !d) return fail(SAM_GPU_EINVAL, "mma_selftest: null array");
  int rc = mlp_ensure(c);
  if (rc) return rc;
  if ((rc = ensure(c.sc[0], 2 * (128 * 16 + 64 * 16) + 256)) || (rc = ensure(c.sc[1], 4 * 128 * 64))) return rc;
  std::vector<__nv_bfloat16> h(128 * 16 + 64 * 16);
  for (int i = 0; i < 128 * 16; ++i) h[i] = __float2bfloat16_rn(a[i]);
  for (int i = 0; i < 64 * 16; ++i) h[128 * 16 + i] = __float2bfloat16_rn(b[i]);
  CK(cudaMemcpyAsync(c.sc[0].p, h.data(), 2 * h.size(), cudaMemcpyHostToDevice, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  const __nv_bfloat16* da = (const __nv_bfloat16*)c.sc[0].p;
  mlp_mma_selftest(da, da + 128 * 16, (float*)c.sc[1].p, c.mlp_err, c.stream);
  CK(cudaMemcpyAsync(d, c.sc[1].p, 4 * 128 * 64, cudaMemcpyDeviceToHost, c.stream));
  return mlp_check_err(c);
}

int sam_gpu_measure_fp64_peak(double* tflops) {
  NEED_CTX();
  if (!tflops) return fail(SAM_GPU_EINVAL, "measure_fp64_peak: null output");
  *tflops = diag_fp64_peak(c.stream);
  return check_launch();
}

// Tile and FFT-schedule autotuner: each pass is timed (CUDA events, best of
// `reps`) with each candidate on the resident state and the fastest is kept.
// The z forward pass updates u and r, and stage 1 recomputes dt, the
// statistics and (dynamic closure) the model coefficient from the state it
// sees, so u, r, p, the scalar state and the coefficient are saved first and
// restored after: the state after the call is the state before it.
int sam_gpu_autotune(int reps) {
  NEED_CTX();
  if (reps < 1) reps = 1;
  const size_t nm = (size_t)c.g.mx * c.g.my * c.g.mz * c.g.lu;
  const size_t bytes = nm * csize(c);
  const size_t pbytes = (size_t)c.g.mx * c.g.my * c.g.mz * csize(c);
  void *su = nullptr, *sr = nullptr, *sp = nullptr, *ss = nullptr;
  CK(cudaMalloc(&su, bytes));
  CK(cudaMalloc(&sr, bytes));
  CK(cudaMalloc(&sp, pbytes));
  CK(cudaMalloc(&ss, sizeof(DevState) + sizeof(double)));
  double* scds = reinterpret_cast<double*>(static_cast<char*>(ss) + sizeof(DevState));
  CK(cudaMemcpyAsync(su, c.U, bytes, cudaMemcpyDeviceToDevice, c.stream));
  CK(cudaMemcpyAsync(sr, c.R, bytes, cudaMemcpyDeviceToDevice, c.stream));
  CK(cudaMemcpyAsync(sp, c.P, pbytes, cudaMemcpyDeviceToDevice, c.stream));
  CK(cudaMemcpyAsync(ss, c.state, sizeof(DevState), cudaMemcpyDeviceToDevice, c.stream));
  if (c.les_cds) CK(cudaMemcpyAsync(scds, c.les_cds, sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  auto time_pass = [&](int p, int nrk = 2) {
    float best = 1e30f;
    for (int r = 0; r < reps + 1; ++r) {
      cudaEventRecord(e0, c.stream);
      if (stage_any(c, nrk, nullptr, p)) return 1e30f;
      cudaEventRecord(e1, c.stream);
      cudaEventSynchronize(e1);
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (r > 0 && ms < best) best = ms;  // the first run warms up
    }
    return best;
  };
  // a candidate replaces the current choice when it is faster by more than
  // `margin`; `both` times stages 1 and 2 together (stage 1 adds vel_max's
  // work to the x pass; stage 3 would advance the time)
  auto tune = [&](int p, int* field, std::initializer_list<int> cands, float margin = 0.0f, bool both = false) {
    auto timed = [&]() { return both ? time_pass(p, 1) + time_pass(p, 2) : time_pass(p); };
    int best_v = *field;
    float best_t = timed();
    for (int v : cands) {
      if (v == best_v) continue;
      const int keep = *field;
      *field = v;
      const float t = timed();
      if (t < best_t * (1.0f - margin)) { best_t = t; best_v = v; }
      else *field = keep;
    }
    *field = best_v;
  };
  tune(0, &c.ty_zi, {4, 8, 16, 32});
  tune(1, &c.tx_yi, {4, 8, 16, 32});
  tune(2, &c.yt_x, {2, 4, 8, 16});
  tune(2, &c.grp_x, {1, 2, 3, 5, 9});
  tune(3, &c.tz_yf, {4, 8, 16, 32});
  tune(4, &c.ty_zf, {1, 2, 4, 8});
  // then the FFT schedule of each pass with length-256 lines (16 x 16
  // registers or compile-time Stockham) with those tiles: the register path
  // stays unless the other is more than 2 % faster over stages 1 and 2
  const int plen[5] = {c.g.nz, c.g.ny, c.g.nx, c.g.ny, c.g.nz};
  for (int p = 0; p < 5; ++p)
    if (plen[p] == 256) tune(p, &c.sched[p], {0, 1}, 0.02f, true);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CK(cudaMemcpyAsync(c.U, su, bytes, cudaMemcpyDeviceToDevice, c.stream));
  CK(cudaMemcpyAsync(c.R, sr, bytes, cudaMemcpyDeviceToDevice, c.stream));
  CK(cudaMemcpyAsync(c.P, sp, pbytes, cudaMemcpyDeviceToDevice, c.stream));
  CK(cudaMemcpyAsync(c.state, ss, sizeof(DevState), cudaMemcpyDeviceToDevice, c.stream));
  if (c.les_cds) CK(cudaMemcpyAsync(c.les_cds, scds, sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  cudaFree(su);
  cudaFree(sr);
  cudaFree(sp);
  cudaFree(ss);
  if (c.gexec) { cudaGraphExecDestroy(c.gexec); c.gexec = nullptr; }
  c.graph_stale = 1;  // recapture with the new tiles
  return check_launch();
}

int sam_gpu_set_fft_schedule(const int* sched5) {
  NEED_CTX();
  if (!sched5) return fail(SAM_GPU_EINVAL, "set_fft_schedule: null array");
  for (int p = 0; p < 5; ++p)
    if (sched5[p] != 0 && sched5[p] != 1 && !(p == 2 && sched5[p] == 2))
      return fail(SAM_GPU_EINVAL, "FFT schedule %d of pass %d", sched5[p], p);
  for (int p = 0; p < 5; ++p) c.sched[p] = sched5[p];
  if (c.gexec) { cudaGraphExecDestroy(c.gexec); c.gexec = nullptr; }
  c.graph_stale = 1;
  return 0;
}

int sam_gpu_fft_schedule(int* out5) {
  NEED_CTX();
  if (!out5) return fail(SAM_GPU_EINVAL, "fft_schedule: null array");
  for (int p = 0; p < 5; ++p) out5[p] = c.sched[p];
  return 0;
}

int sam_gpu_tiles(int* out6) {
  NEED_CTX();
  if (!out6) return fail(SAM_GPU_EINVAL, "tiles: null array");
  out6[0] = c.ty_zi; out6[1] = c.tx_yi; out6[2] = c.yt_x; out6[3] = c.grp_x; out6[4] = c.tz_yf; out6[5] = c.ty_zf;
  return 0;
}

int sam_gpu_set_tiles(const int* in6) {
  NEED_CTX();
  if (!in6) return fail(SAM_GPU_EINVAL, "set_tiles: null array");
  for (int p = 0; p < 6; ++p)
    if (in6[p] < 1 || in6[p] > 64) return fail(SAM_GPU_EINVAL, "set_tiles: tile %d of entry %d", in6[p], p);
  if (in6[2] % 2) return fail(SAM_GPU_EINVAL, "set_tiles: x-pass rows %d (row pairs: even)", in6[2]);
  c.ty_zi = in6[0]; c.tx_yi = in6[1]; c.yt_x = in6[2]; c.grp_x = in6[3]; c.tz_yf = in6[4]; c.ty_zf = in6[5];
  if (c.gexec) { cudaGraphExecDestroy(c.gexec); c.gexec = nullptr; }
  c.graph_stale = 1;
  return 0;
}

int sam_gpu_profile_stage(int nrk, int reps, float* ms5) {
  NEED_CTX();
  if (nrk < 1 || nrk > c.cfg.nrk_max || reps < 1 || !ms5) return fail(SAM_GPU_EINVAL, "profile_stage: bad arguments");
  cudaEvent_t ev[6];
  for (auto& e : ev) CK(cudaEventCreate(&e));
  for (int p = 0; p < 5; ++p) ms5[p] = 0.0f;
  int rc = 0;
  for (int r = 0; r < reps && !rc; ++r) {
    rc = stage_any(c, nrk, ev);
    if (rc) break;
    CK(cudaEventSynchronize(ev[5]));
    for (int p = 0; p < 5; ++p) {
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, ev[p], ev[p + 1]);
      ms5[p] += ms / (float)reps;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (rc) return rc;
  return check_launch();
}

// ---------------------------------------------------------- initial fields

static int init_finish(Ctx& c, double2* tmp) {
  const Grid& g = c.g;
  const size_t nm = (size_t)g.mx * g.my * g.mz * g.lu;
  if (c.cfg.precision != 64) state_from_fp64(c, tmp, c.U, (long long)nm);
  CK(cudaMemsetAsync(c.R, 0, csize(c) * nm, c.stream));
  return sync_stream(c);
}

static int init_target(Ctx& c, double2** out) {
  const Grid& g = c.g;
  const size_t nm = (size_t)g.mx * g.my * g.mz * g.lu;
  if (c.cfg.precision != 64) {
    int rc = ensure(c.sc[0], nm * 16);
    if (rc) return rc;
    *out = (double2*)c.sc[0].p;
  } else {
    *out = (double2*)c.U;
  }
  return 0;
}

int sam_gpu_init_taylor_green(void) {
  NEED_CTX();
  if (c.g.kx < 1 || c.g.ky < 1 || c.g.kz < 1) return fail(SAM_GPU_EINVAL, "grid too small for Taylor-Green");
  double2* u;
  int rc = init_target(c, &u);
  if (rc) return rc;
  fields_init_tg(u, c.g, c.stream);
  return init_finish(c, u);
}

int sam_gpu_init_random(unsigned long long seed, int kind_u, double flct_u, int kind_t, double flct_t) {
  NEED_CTX();
  double2* u;
  int rc = init_target(c, &u);
  if (rc) return rc;
  fields_init_random(u, c.g, seed, kind_u, flct_u, kind_t, flct_t, c.stream);
  return init_finish(c, u);
}

int sam_gpu_init_packet(unsigned long long seed, int kx0, int ky0, int kz0, double sigma, double amplitude,
                        double noise) {
  NEED_CTX();
  double2* u;
  int rc = init_target(c, &u);
  if (rc) return rc;
  fields_init_packet(u, c.g, seed, kx0, ky0, kz0, sigma, amplitude, noise, c.cfg.xl, c.cfg.yl, c.cfg.zl,
                     c.cfg.buoy_fac_z, c.cfg.lapse, c.stream);
  return init_finish(c, u);
}

// ------------------------------------------------------------- diagnostics

// The state the diagnostics read: U and R themselves in the FP64 and FP32
// forms; FP64 copies (scratch 1 and 2) in the double-float form, whose
// diagnostics then run the FP64 kernels (prec).
static int diag_state(Ctx& c, bool with_r, void** u, const void** r, int* prec) {
  *u = c.U;
  if (r) *r = c.R;
  *prec = c.cfg.precision;
  if (c.cfg.precision != kPrecDD) return 0;
  const long long nm = (long long)c.g.mx * c.g.my * c.g.mz * c.g.lu;
  int rc;
  if ((rc = ensure(c.sc[1], (size_t)nm * 16))) return rc;
  state_to_fp64(c, c.U, (double2*)c.sc[1].p, nm);
  *u = c.sc[1].p;
  if (with_r) {
    if ((rc = ensure(c.sc[2], (size_t)nm * 16))) return rc;
    state_to_fp64(c, c.R, (double2*)c.sc[2].p, nm);
    *r = c.sc[2].p;
  }
  *prec = 64;
  return 0;
}

int sam_gpu_spectra(double* out) {
  NEED_CTX();
  int rc = ensure(c.sc[3], sizeof(double) * ((size_t)5 * c.lm + 8) * 1024);
  if (rc) return rc;
  double e_cl = 0.0;
  if (c.cfg.i_les) {
    if ((rc = sam_gpu_cl_energy(&e_cl))) return rc;
  }
  void* u;
  const void* r;
  int prec;
  if ((rc = diag_state(c, true, &u, &r, &prec))) return rc;
  DiagArgs d = diag_args(c.g, c.lm, c.nx2, c.k_cl, c.cfg.vis, c.cfg.i_les, e_cl, prec);
  diag_spectra(d, u, r, (double*)c.sc[3].p, out, c.stream);
  return sync_stream(c);
}

int sam_gpu_div_check(double* out4) {
  NEED_CTX();
  int rc = ensure(c.sc[3], sizeof(double) * 8 * 1024);
  if (rc) return rc;
  void* u;
  int prec;
  if ((rc = diag_state(c, false, &u, nullptr, &prec))) return rc;
  DiagArgs d = diag_args(c.g, c.lm, c.nx2, c.k_cl, c.cfg.vis, c.cfg.i_les, 0.0, prec);
  diag_div_check(d, u, (double*)c.sc[3].p, out4, c.stream);
  return sync_stream(c);
}

int sam_gpu_cl_energy(double* e_cl) {
  NEED_CTX();
  int rc = ensure(c.sc[3], sizeof(double) * 8 * 1024);
  if (rc) return rc;
  void* u;
  int prec;
  if ((rc = diag_state(c, false, &u, nullptr, &prec))) return rc;
  DiagArgs d = diag_args(c.g, c.lm, c.nx2, c.k_cl, c.cfg.vis, c.cfg.i_les, 0.0, prec);
  diag_cl_energy(d, u, (double*)c.sc[3].p, e_cl, c.stream);
  return sync_stream(c);
}

int sam_gpu_force(const double* ek_0, int k_force) {
  NEED_CTX();
  if (!ek_0 || k_force < 1 || k_force >= 64 || k_force >= c.lm)
    return fail(SAM_GPU_EINVAL, "force: k_force must be in 1..min(63, Lm-1)");
  int rc = ensure(c.sc[3], sizeof(double) * 64);
  if (rc) return rc;
  CK(cudaMemcpyAsync(c.sc[3].p, ek_0, sizeof(double) * (k_force + 1), cudaMemcpyHostToDevice, c.stream));
  void* u;
  int prec;
  if ((rc = diag_state(c, false, &u, nullptr, &prec))) return rc;
  DiagArgs d = diag_args(c.g, c.lm, c.nx2, c.k_cl, c.cfg.vis, c.cfg.i_les, 0.0, prec);
  diag_force(d, u, (const double*)c.sc[3].p, k_force, c.stream);
  // the double-float form rescaled an FP64 copy: back into the state
  if (u != c.U) state_from_fp64(c, (const double2*)u, c.U, (long long)c.g.mx * c.g.my * c.g.mz * c.g.lu);
  return sync_stream(c);
}

// ------------------------------------------------------------- restart files
// vel.NNNNNN (write_field.f:12-30): for each field n and kx index ii a record
// of Nz_min x Ny_min complex128 at offset ((n-1) Nx_min + ii-1) * record, i.e.
// the fields in exactly the resident (field, kx, ky, kz) order.

static int resident_fp64(Ctx& c, const double2** out) {
  const size_t nm = (size_t)c.g.mx * c.g.my * c.g.mz * c.g.lu;
  if (c.cfg.precision == 64) {
    *out = (const double2*)c.U;
    return 0;
  }
  int rc = ensure(c.sc[1], nm * 16);
  if (rc) return rc;
  state_to_fp64(c, c.U, (double2*)c.sc[1].p, (long long)nm);
  *out = (const double2*)c.sc[1].p;
  return 0;
}

int sam_gpu_write_field(const char* fname) {
  NEED_CTX();
  if (!fname) return fail(SAM_GPU_EINVAL, "write_field: null file name");
  const size_t bytes = (size_t)c.g.mx * c.g.my * c.g.mz * c.g.lu * 16;
  const double2* src;
  int rc = resident_fp64(c, &src);
  if (rc) return rc;
  std::vector<char> host(bytes);
  CK(cudaMemcpyAsync(host.data(), src, bytes, cudaMemcpyDeviceToHost, c.stream));
  if ((rc = sync_stream(c))) return rc;
  FILE* f = fopen(fname, "wb");
  if (!f) return fail(SAM_GPU_EINVAL, "write_field: cannot open %s", fname);
  const size_t w = fwrite(host.data(), 1, bytes, f);
  fclose(f);
  if (w != bytes) return fail(SAM_GPU_EINVAL, "write_field: short write to %s", fname);
  return 0;
}

int sam_gpu_read_field(const char* fname) {
  NEED_CTX();
  if (!fname) return fail(SAM_GPU_EINVAL, "read_field: null file name");
  const size_t nm = (size_t)c.g.mx * c.g.my * c.g.mz * c.g.lu;
  const size_t expect = nm * 16;
  FILE* f = fopen(fname, "rb");
  if (!f) return fail(SAM_GPU_EINVAL, "read_field: cannot open %s", fname);
  fseek(f, 0, SEEK_END);
  const long found = ftell(f);
  fseek(f, 0, SEEK_SET);
  if (found < 0 || (size_t)found != expect) {  // read_field.f:26-32
    fclose(f);
    return fail(SAM_GPU_EINVAL, "read_field: vel file is not of correct size (expect %zu, found %ld)", expect, found);
  }
  std::vector<char> host(expect);
  const size_t r = fread(host.data(), 1, expect, f);
  fclose(f);
  if (r != expect) return fail(SAM_GPU_EINVAL, "read_field: short read from %s", fname);
  int rc;
  void* dst = c.U;
  if (c.cfg.precision != 64) {
    if ((rc = ensure(c.sc[0], expect))) return rc;
    dst = c.sc[0].p;
  }
  CK(cudaMemcpyAsync(dst, host.data(), expect, cudaMemcpyHostToDevice, c.stream));
  if (c.cfg.precision != 64) state_from_fp64(c, (const double2*)dst, c.U, (long long)nm);
  CK(cudaMemsetAsync(c.R, 0, csize(c) * nm, c.stream));
  return sync_stream(c);
}

// header.NNNNNN (write_header.f:27-31): one "label value" line per
// parameter; the restart-fixed ones (set_labels.f:29-57: box and grid, the
// stratification switch) must agree on reading (read_header.f:25-38), and
// time and dt are restored (assign_run_time.f).
int sam_gpu_write_header(const char* fname, int nt) {
  NEED_CTX();
  DevState st;
  CK(cudaMemcpyAsync(&st, c.state, sizeof(st), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  FILE* f = fopen(fname, "w");
  if (!f) return fail(SAM_GPU_EINVAL, "write_header: cannot open %s", fname);
  const sam_gpu_config& k = c.cfg;
  fprintf(f, " xL %.17g\n yL %.17g\n zL %.17g\n c_smag %.17g\n dt0 %.17g\n cfl0 %.17g\n vis %.17g\n pr %.17g\n",
          k.xl, k.yl, k.zl, k.c_smag, k.dt0, k.cfl0, k.vis, k.pr);
  fprintf(f, " Nx %d\n Ny %d\n Nz %d\n i_strat %d\n i_les %d\n i_cfl %d\n nrk_max %d\n n_dealias %d\n", k.nx, k.ny,
          k.nz, k.i_strat, k.i_les, k.i_cfl, k.nrk_max, k.n_dealias);
  fprintf(f, " time %.17g\n dt %.17g\n t_stat %.17g\n nt %d\n n_frame_p %d\n n_hist %d\n", st.time, st.dt, 0.0, nt, 0,
          0);
  fclose(f);
  return 0;
}

int sam_gpu_read_header(const char* fname, int* nt) {
  NEED_CTX();
  FILE* f = fopen(fname, "r");
  if (!f) return fail(SAM_GPU_EINVAL, "read_header: cannot open %s", fname);
  char label[64];
  double v;
  double time = 0.0, dt = c.cfg.dt0;
  int got_nt = 0, bad = 0;
  char which[64] = "";
  const sam_gpu_config& k = c.cfg;
  while (fscanf(f, "%63s %lf", label, &v) == 2) {
    std::string s(label);
    for (auto& ch : s) ch = (char)tolower(ch);
    auto fixed = [&](const char* nm, double have) {
      if (s == nm && fabs(v - have) > 1.0e-12) { bad = 1; snprintf(which, sizeof(which), "%s", nm); }
    };
    fixed("xl", k.xl); fixed("yl", k.yl); fixed("zl", k.zl);
    fixed("nx", k.nx); fixed("ny", k.ny); fixed("nz", k.nz); fixed("i_strat", k.i_strat);
    if (s == "time") time = v;
    else if (s == "dt") dt = v;
    else if (s == "nt") got_nt = (int)v;
  }
  fclose(f);
  if (bad) return fail(SAM_GPU_EINVAL, "read_header: parameter %s differs between the header and the configuration", which);
  if (nt) *nt = got_nt;
  DevState st;
  CK(cudaMemcpyAsync(&st, c.state, sizeof(st), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  st.time = time;
  st.dt = dt;
  CK(cudaMemcpyAsync(c.state, &st, sizeof(st), cudaMemcpyHostToDevice, c.stream));
  return sync_stream(c);
}

int sam_gpu_x_deriv(const double* u, double* du, double*) {
  NEED_CTX();
  if (!u || !du) return fail(SAM_GPU_EINVAL, "x_deriv: null array");
  const size_t n = (size_t)c.g.nx * c.g.ny;
  int rc;
  if ((rc = ensure(c.sc[0], n * 8)) || (rc = ensure(c.sc[1], n * 8))) return rc;
  CK(cudaMemcpyAsync(c.sc[0].p, u, n * 8, cudaMemcpyHostToDevice, c.stream));
  diag_deriv(c.g, 0, c.px.d, c.px.tw64, c.px.h, (const double*)c.sc[0].p, (double*)c.sc[1].p, c.stream);
  CK(cudaMemcpyAsync(du, c.sc[1].p, n * 8, cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

// ------------------------------------------------ subgrid models, get_mean

int sam_gpu_filter(const double* f_bar, double* f_hat, int n_var) {
  NEED_CTX();
  if (!f_bar || !f_hat || n_var < 1) return fail(SAM_GPU_EINVAL, "filter: bad arguments");
  const size_t pl = (size_t)(c.g.nx + 2) * (c.g.ny + 2);
  int rc;
  if ((rc = ensure(c.sc[0], pl * n_var * 3 * 8)) || (rc = ensure(c.sc[1], pl * n_var * 8))) return rc;
  CK(cudaMemcpyAsync(c.sc[0].p, f_bar, pl * n_var * 3 * 8, cudaMemcpyHostToDevice, c.stream));
  les_filter((const double*)c.sc[0].p, (double*)c.sc[1].p, c.g.nx, c.g.ny, n_var, c.stream);
  CK(cudaMemcpyAsync(f_hat, c.sc[1].p, pl * n_var * 8, cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}


int sam_gpu_sm(const double* u, double*, double*, double* vt) {
  NEED_CTX();
  if (!u || !vt) return fail(SAM_GPU_EINVAL, "sm: null array");
  const Grid& g = c.g;
  const size_t vol = (size_t)(g.nx + 2) * (g.ny + 2) * (g.nz + 2);
  const size_t n = (size_t)g.nx * g.ny * g.nz;
  int rc;
  if ((rc = ensure(c.sc[0], vol * 3 * 8)) || (rc = ensure(c.sc[1], vol * 8)) || (rc = ensure(c.sc[2], n * 3 * 8)))
    return rc;
  double dxi, dyi, dzi, dsq;
  grid_spacing(c, dxi, dyi, dzi, dsq);
  CK(cudaMemcpyAsync(c.sc[0].p, u, vol * 3 * 8, cudaMemcpyHostToDevice, c.stream));
  CK(cudaMemsetAsync(c.sc[1].p, 0, vol * 8, c.stream));
  les_sm((const double*)c.sc[0].p, (double*)c.sc[2].p, (double*)c.sc[1].p, g.nx, g.ny, g.nz, c.cfg.c_smag * dsq, dxi,
         dyi, dzi, c.stream);
  CK(cudaMemcpyAsync(vt, c.sc[1].p, vol * 8, cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

int sam_gpu_dm(const double* u, double*, double*, double*, double*, double*, double*, double*, double*, double* vt,
               double* c_delta_sq) {
  NEED_CTX();
  if (!u || !vt) return fail(SAM_GPU_EINVAL, "dm: null array");
  const Grid& g = c.g;
  const size_t vol = (size_t)(g.nx + 2) * (g.ny + 2) * (g.nz + 2);
  const size_t n = (size_t)g.nx * g.ny * g.nz;
  const int nb = les_dm_blocks(g.nx, g.ny, g.nz);
  int rc;
  if ((rc = ensure(c.sc[0], vol * 3 * 8)) || (rc = ensure(c.sc[1], vol * 8)) ||
      (rc = ensure(c.sc[2], n * 22 * 8)) || (rc = ensure(c.sc[3], (2 * (size_t)nb + 8) * 8)))
    return rc;
  double dxi, dyi, dzi, dsq;
  grid_spacing(c, dxi, dyi, dzi, dsq);
  double* ub = (double*)c.sc[2].p;
  double* q = ub + 3 * n;
  double* part = (double*)c.sc[3].p;
  double* cds = part + 2 * nb;
  CK(cudaMemcpyAsync(c.sc[0].p, u, vol * 3 * 8, cudaMemcpyHostToDevice, c.stream));
  CK(cudaMemsetAsync(c.sc[1].p, 0, vol * 8, c.stream));
  les_dm((const double*)c.sc[0].p, ub, q, part, cds, (double*)c.sc[1].p, g.nx, g.ny, g.nz, 4.0, dxi, dyi, dzi,
         c.stream);
  CK(cudaMemcpyAsync(vt, c.sc[1].p, vol * 8, cudaMemcpyDeviceToHost, c.stream));
  if (c_delta_sq) CK(cudaMemcpyAsync(c_delta_sq, cds, 8, cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

int sam_gpu_get_mean(double* u, int i_symm, int i_remove, double* u_mean, double* jump, double*) {
  NEED_CTX();
  const Grid& g = c.g;
  if (!u || !u_mean || !jump) return fail(SAM_GPU_EINVAL, "get_mean: null array");
  if (i_symm != 0) return fail(SAM_GPU_EUNSUPPORTED, "get_mean: only the periodic branch (i_symm=0) is supported");
  if (g.nz < 3) return fail(SAM_GPU_EINVAL, "get_mean: Nz must be >= 3");
  int rc;
  if ((rc = ensure(c.sc[0], ((size_t)g.mz * 2 + (size_t)g.nz + 8) * 8))) return rc;
  double2* col = (double2*)c.sc[0].p;
  double* dmean = (double*)(col + g.mz);
  double* djump = dmean + g.nz;
  CK(cudaMemcpyAsync(col, u, (size_t)g.mz * 16, cudaMemcpyHostToDevice, c.stream));
  les_get_mean(col, g.mz, g.kz, g.nz, i_remove, c.pz.d, c.pz.tw64, c.pz.h, dmean, djump, c.stream);
  CK(cudaMemcpyAsync(u, col, (size_t)g.mz * 16, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(u_mean, dmean, (size_t)g.nz * 8, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(jump, djump, 8, cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

int sam_gpu_planes(const int* k_xy, int n_xy, const int* j_xz, int n_xz, const int* i_yz, int n_yz, double* xy,
                   double* xz, double* yz, double* mean) {
  NEED_CTX();
  const Grid& g = c.g;
  if (n_xy < 0 || n_xz < 0 || n_yz < 0 || n_xy > SAM_GPU_MAX_PLANES || n_xz > SAM_GPU_MAX_PLANES ||
      n_yz > SAM_GPU_MAX_PLANES)
    return fail(SAM_GPU_EINVAL, "planes: plane counts must be 0..%d", SAM_GPU_MAX_PLANES);
  if ((n_xy && (!k_xy || !xy)) || (n_xz && (!j_xz || !xz)) || (n_yz && (!i_yz || !yz)))
    return fail(SAM_GPU_EINVAL, "planes: null plane list or output array");
  if (g.nz < 3) return fail(SAM_GPU_EINVAL, "planes: Nz must be >= 3 (get_mean)");
  PlaneSel sel{};
  sel.n_xy = n_xy; sel.n_xz = n_xz; sel.n_yz = n_yz;
  for (int m = 0; m < n_xy; ++m) {
    if (k_xy[m] < 1 || k_xy[m] > g.nz) return fail(SAM_GPU_EINVAL, "planes: k_xy(%d) = %d outside 1..%d", m + 1, k_xy[m], g.nz);
    sel.k_xy[m] = k_xy[m] - 1;
  }
  for (int m = 0; m < n_xz; ++m) {
    if (j_xz[m] < 1 || j_xz[m] > g.ny) return fail(SAM_GPU_EINVAL, "planes: j_xz(%d) = %d outside 1..%d", m + 1, j_xz[m], g.ny);
    sel.j_xz[m] = j_xz[m] - 1;
  }
  for (int m = 0; m < n_yz; ++m) {
    if (i_yz[m] < 1 || i_yz[m] > g.nx) return fail(SAM_GPU_EINVAL, "planes: i_yz(%d) = %d outside 1..%d", m + 1, i_yz[m], g.nx);
    sel.i_yz[m] = i_yz[m] - 1;
  }
  if (c.cfg.precision == kPrecDD) return fail(SAM_GPU_EUNSUPPORTED, "planes: not in the double-float form");
  const int rc = c.cfg.precision == 32 ? planes_impl<float>(c, sel, xy, xz, yz, mean)
                                       : planes_impl<double>(c, sel, xy, xz, yz, mean);
  if (rc) return rc;
  return sync_stream(c);
}

int sam_gpu_y_deriv(const double* u, double* du, double*) {
  NEED_CTX();
  if (!u || !du) return fail(SAM_GPU_EINVAL, "y_deriv: null array");
  const size_t n = (size_t)c.g.nx * c.g.ny;
  int rc;
  if ((rc = ensure(c.sc[0], n * 8)) || (rc = ensure(c.sc[1], n * 8))) return rc;
  CK(cudaMemcpyAsync(c.sc[0].p, u, n * 8, cudaMemcpyHostToDevice, c.stream));
  diag_deriv(c.g, 1, c.py.d, c.py.tw64, c.py.h, (const double*)c.sc[0].p, (double*)c.sc[1].p, c.stream);
  CK(cudaMemcpyAsync(du, c.sc[1].p, n * 8, cudaMemcpyDeviceToHost, c.stream));
  return sync_stream(c);
}

}  // extern "C"
