"""Python host-side mirror of the SAM routines on the GB300 library.

A thin ctypes layer over libsam_gpu.so (C ABI in include/sam_gpu.h).  Method
names and argument meanings follow the reference's Fortran subroutines
(z_trans_b, x2z_decomp, xy_trans_b, rhs, ...) and arrays use the reference's
column-major layouts, so code written against the reference reads the same.
There is no CPU path: if the library or a GPU is missing, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# SAM_GPU_LIB selects another build of the same library (e.g. a tuning variant)
LIB_PATH = os.environ.get("SAM_GPU_LIB", os.path.join(HERE, "_lib", "libsam_gpu.so"))

SAM_GPU_OK = 0
ERRORS = {-1: "EINVAL", -2: "ENOTINIT", -3: "EUNSUPPORTED", -4: "ECUDA", -5: "ENONFINITE"}

EXPORTS = [
    "sam_gpu_init", "sam_gpu_finalize", "sam_gpu_dims", "sam_gpu_set_tstep", "sam_gpu_get_stats",
    "sam_gpu_set_stream", "sam_gpu_error_string", "sam_gpu_z_trans_b", "sam_gpu_x2z_decomp",
    "sam_gpu_xy_trans_b", "sam_gpu_xy_trans_f", "sam_gpu_z2x_decomp", "sam_gpu_z_trans_f", "sam_gpu_vel_max",
    "sam_gpu_rhs", "sam_gpu_x_deriv", "sam_gpu_y_deriv", "sam_gpu_upload", "sam_gpu_download", "sam_gpu_stage",
    "sam_gpu_step", "sam_gpu_spectra", "sam_gpu_div_check", "sam_gpu_cl_energy", "sam_gpu_init_taylor_green",
    "sam_gpu_init_random", "sam_gpu_init_packet", "sam_gpu_profile_stage", "sam_gpu_measure_fp64_peak",
    "sam_gpu_vel_max_noalloc", "sam_gpu_filter", "sam_gpu_sm", "sam_gpu_dm", "sam_gpu_get_mean",
    "sam_gpu_force", "sam_gpu_write_field", "sam_gpu_read_field", "sam_gpu_write_header", "sam_gpu_read_header",
    "sam_gpu_autotune", "sam_gpu_tiles", "sam_gpu_set_tiles", "sam_gpu_set_fft_schedule", "sam_gpu_fft_schedule",
    "sam_gpu_planes",
    "sam_gpu_set_forcing", "sam_gpu_set_les", "sam_gpu_les_coef",
    "sam_gpu_mlp_set", "sam_gpu_mlp_get", "sam_gpu_mlp_forward", "sam_gpu_mlp_grad", "sam_gpu_mlp_train",
    "sam_gpu_mlp_set_backward",
    "sam_gpu_mma_selftest", "sam_gpu_box_filter", "sam_gpu_closure_inputs",
    "sam_gpu_ensemble_create", "sam_gpu_ensemble_select", "sam_gpu_ensemble_step", "sam_gpu_ensemble_destroy",
    "sam_gpu_ensemble_set_persistent", "sam_gpu_ensemble_persistent_members",
]

TILE_KEYS = ("z_inv_rows", "y_inv_cols", "x_rows", "x_group", "y_fwd_planes", "z_fwd_rows")
MLP_PARAMS = 5122
MLP_FEATURES = 12


class SamGpuError(RuntimeError):
    pass


class Config(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("n_dealias", C.c_int), ("i_strat", C.c_int), ("i_cfl", C.c_int),
        ("nrk_max", C.c_int), ("rot_sav", C.c_int), ("i_les", C.c_int), ("precision", C.c_int),
        ("xl", C.c_double), ("yl", C.c_double), ("zl", C.c_double),
        ("vis", C.c_double), ("pr", C.c_double),
        ("dt0", C.c_double), ("cfl0", C.c_double),
        ("buoy_fac_x", C.c_double), ("buoy_fac_z", C.c_double), ("lapse", C.c_double),
        ("cos_theta", C.c_double), ("sin_theta", C.c_double),
        ("c_smag", C.c_double),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("time", C.c_double), ("dt", C.c_double),
        ("u_avg", C.c_double * 4), ("u_var", C.c_double * 4), ("u_max", C.c_double * 4),
        ("energy", C.c_double), ("cfl_x", C.c_double), ("cfl_y", C.c_double), ("cfl_z", C.c_double),
        ("nonfinite", C.c_int), ("pad", C.c_int),
    ]


_lib = None


def load_library(path: str = LIB_PATH):
    """Load libsam_gpu.so (build it with sam_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise SamGpuError(f"{path} is missing: run sam_gb300.build.build() (there is no CPU fallback)")
    lib = C.CDLL(path)
    P = C.c_void_p
    lib.sam_gpu_init.argtypes = [C.POINTER(Config)]
    lib.sam_gpu_dims.argtypes = [P]
    lib.sam_gpu_set_tstep.argtypes = [C.c_int, C.c_double, C.c_double]
    lib.sam_gpu_get_stats.argtypes = [C.POINTER(Stats)]
    lib.sam_gpu_set_stream.argtypes = [P]
    lib.sam_gpu_error_string.restype = C.c_char_p
    lib.sam_gpu_z_trans_b.argtypes = [P, P, C.c_int, P, P, P, P]
    lib.sam_gpu_x2z_decomp.argtypes = [P, P, C.c_int, P]
    lib.sam_gpu_xy_trans_b.argtypes = [P, P, C.c_int, P]
    lib.sam_gpu_xy_trans_f.argtypes = [P, P, C.c_int, P]
    lib.sam_gpu_z2x_decomp.argtypes = [P, P, C.c_int, P]
    lib.sam_gpu_z_trans_f.argtypes = [P, C.c_int, P, P, P]
    lib.sam_gpu_vel_max.argtypes = [P, P]
    lib.sam_gpu_rhs.argtypes = [P, P, P, P, P]
    lib.sam_gpu_x_deriv.argtypes = [P, P, P]
    lib.sam_gpu_y_deriv.argtypes = [P, P, P]
    lib.sam_gpu_upload.argtypes = [P]
    lib.sam_gpu_download.argtypes = [P, P]
    lib.sam_gpu_stage.argtypes = [C.c_int]
    lib.sam_gpu_step.argtypes = [C.c_int]
    lib.sam_gpu_spectra.argtypes = [P]
    lib.sam_gpu_div_check.argtypes = [P]
    lib.sam_gpu_cl_energy.argtypes = [P]
    lib.sam_gpu_init_random.argtypes = [C.c_ulonglong, C.c_int, C.c_double, C.c_int, C.c_double]
    lib.sam_gpu_init_packet.argtypes = [C.c_ulonglong, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                        C.c_double]
    lib.sam_gpu_profile_stage.argtypes = [C.c_int, C.c_int, P]
    lib.sam_gpu_measure_fp64_peak.argtypes = [C.POINTER(C.c_double)]
    lib.sam_gpu_vel_max_noalloc.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, P, P]
    lib.sam_gpu_filter.argtypes = [P, P, C.c_int]
    lib.sam_gpu_sm.argtypes = [P, P, P, P]
    lib.sam_gpu_dm.argtypes = [P] * 11
    lib.sam_gpu_get_mean.argtypes = [P, C.c_int, C.c_int, P, P, P]
    lib.sam_gpu_autotune.argtypes = [C.c_int]
    lib.sam_gpu_tiles.argtypes = [P]
    lib.sam_gpu_set_fft_schedule.argtypes = [P]
    lib.sam_gpu_set_tiles.argtypes = [P]
    lib.sam_gpu_fft_schedule.argtypes = [P]
    lib.sam_gpu_set_forcing.argtypes = [C.c_ulonglong, C.c_double, C.c_double, C.c_double, C.POINTER(C.c_int)]
    lib.sam_gpu_set_les.argtypes = [C.c_int, C.c_double, C.c_double]
    lib.sam_gpu_mlp_set.argtypes = [P, C.c_int]
    lib.sam_gpu_mlp_get.argtypes = [P, C.c_int]
    lib.sam_gpu_mlp_forward.argtypes = [P, C.c_longlong, P]
    lib.sam_gpu_mlp_grad.argtypes = [P, P, C.c_longlong, P, P]
    lib.sam_gpu_mlp_train.argtypes = [P, P, C.c_longlong, C.c_int, C.c_int, C.c_float, P]
    lib.sam_gpu_mlp_set_backward.argtypes = [C.c_int]
    lib.sam_gpu_mma_selftest.argtypes = [P, P, P]
    lib.sam_gpu_box_filter.argtypes = [C.c_int, P]
    lib.sam_gpu_ensemble_create.argtypes = [P, C.c_int]
    lib.sam_gpu_ensemble_select.argtypes = [C.c_int]
    lib.sam_gpu_ensemble_step.argtypes = [C.c_int]
    lib.sam_gpu_ensemble_set_persistent.argtypes = [C.c_int]
    lib.sam_gpu_ensemble_persistent_members.argtypes = [C.POINTER(C.c_int)]
    lib.sam_gpu_closure_inputs.argtypes = [P, P]
    lib.sam_gpu_les_coef.argtypes = [C.POINTER(C.c_double)]
    lib.sam_gpu_planes.argtypes = [P, C.c_int, P, C.c_int, P, C.c_int, P, P, P, P]
    lib.sam_gpu_force.argtypes = [P, C.c_int]
    lib.sam_gpu_write_field.argtypes = [C.c_char_p]
    lib.sam_gpu_read_field.argtypes = [C.c_char_p]
    lib.sam_gpu_write_header.argtypes = [C.c_char_p, C.c_int]
    lib.sam_gpu_read_header.argtypes = [C.c_char_p, C.POINTER(C.c_int)]
    _lib = lib
    return lib


def _p(a):
    if a is None:
        return None
    assert isinstance(a, np.ndarray)
    assert a.flags["F_CONTIGUOUS"] or a.ndim <= 1, "arrays must be Fortran-ordered"
    return a.ctypes.data_as(C.c_void_p)


def reference_config(nx, ny, nz, *, i_strat=0, n_dealias=1, i_cfl=0, nrk_max=3, xl=2 * np.pi, yl=2 * np.pi,
                     zl=2 * np.pi, vis=0.0, pr=1.0, dt0=0.01, cfl0=0.5, grav=0.0, to=1.0, lapse0=0.0,
                     rot_sav=0, i_les=0, precision=64, cos_theta=1.0, sin_theta=0.0, c_smag=0.01, **_):
    """Config values derived as init.f and initial_field.f derive them:
    buoy_fac_z = grav/To when stratified (initial_field.f:159-161) and
    lapse = lapse0 (initial_field.f:37)."""
    return dict(nx=nx, ny=ny, nz=nz, n_dealias=n_dealias, i_strat=i_strat, i_cfl=i_cfl, nrk_max=nrk_max,
                rot_sav=rot_sav, i_les=i_les, precision=precision, xl=xl, yl=yl, zl=zl, vis=vis, pr=pr, dt0=dt0,
                cfl0=cfl0, buoy_fac_x=0.0, buoy_fac_z=(grav / to if i_strat else 0.0),
                lapse=(lapse0 if i_strat else 0.0), cos_theta=cos_theta, sin_theta=sin_theta, c_smag=c_smag)


class SamGpu:
    """The device context (one per process; the reference's COMMON state)."""

    _live = None

    def __init__(self, **cfg):
        lib = load_library()
        if SamGpu._live is not None:
            SamGpu._live.close()
        self.cfg = Config()
        defaults = dict(n_dealias=1, i_strat=0, i_cfl=0, nrk_max=3, rot_sav=0, i_les=0, precision=64,
                        xl=2 * np.pi, yl=2 * np.pi, zl=2 * np.pi, vis=0.0, pr=1.0, dt0=0.01, cfl0=0.5,
                        buoy_fac_x=0.0, buoy_fac_z=0.0, lapse=0.0, cos_theta=1.0, sin_theta=0.0, c_smag=0.01)
        defaults.update(cfg)
        for k, v in defaults.items():
            setattr(self.cfg, k, v)
        self._check(lib.sam_gpu_init(C.byref(self.cfg)), "sam_gpu_init")
        SamGpu._live = self
        d = np.zeros(11, dtype=np.int32)
        self._check(lib.sam_gpu_dims(d.ctypes.data_as(C.c_void_p)), "sam_gpu_dims")
        (self.nx_min, self.ny_min, self.nz_min, self.nze, self.lu, self.lr, self.kx_max, self.ky_max,
         self.kz_max, self.lm, self.nx2) = [int(x) for x in d]
        self.nx, self.ny, self.nz = self.cfg.nx, self.cfg.ny, self.cfg.nz

    def _check(self, rc, what):
        if rc != SAM_GPU_OK:
            msg = load_library().sam_gpu_error_string().decode(errors="replace")
            raise SamGpuError(f"{what} failed ({ERRORS.get(rc, rc)}): {msg}")

    def close(self):
        if SamGpu._live is self:
            load_library().sam_gpu_finalize()
            SamGpu._live = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- arrays in the reference layouts
    def wave(self, n):
        return np.zeros((self.nze, self.ny_min, self.nx_min, n), dtype=np.complex128, order="F")

    def zblocks(self, n):
        return np.zeros((self.ny_min, self.nx_min, self.nze, n), dtype=np.complex128, order="F")

    def xyplanes(self, n):
        return np.zeros((self.ny, self.nx2, self.nz, n), dtype=np.complex128, order="F")

    def phys(self, n):
        return np.zeros((self.nx, self.ny, self.nz, n), dtype=np.float64, order="F")

    # ---- state
    def set_tstep(self, nrk, dt, time):
        self._check(load_library().sam_gpu_set_tstep(nrk, dt, time), "set_tstep")

    def stats(self):
        s = Stats()
        self._check(load_library().sam_gpu_get_stats(C.byref(s)), "get_stats")
        return dict(time=s.time, dt=s.dt, u_avg=np.array(s.u_avg[:]), u_var=np.array(s.u_var[:]),
                    u_max=np.array(s.u_max[:]), energy=s.energy, cfl_x=s.cfl_x, cfl_y=s.cfl_y, cfl_z=s.cfl_z,
                    nonfinite=s.nonfinite)

    def set_stream(self, stream_handle):
        self._check(load_library().sam_gpu_set_stream(C.c_void_p(stream_handle)), "set_stream")

    # ---- per-routine drop-ins
    def z_trans_b(self, u1, n_var, isymm=None):
        u2 = self.zblocks(n_var)
        iv = np.zeros(n_var, dtype=np.int32) if isymm is None else np.asarray(isymm, dtype=np.int32)
        self._check(load_library().sam_gpu_z_trans_b(_p(u1), _p(u2), n_var, _p(iv), None, None, None), "z_trans_b")
        return u2

    def x2z_decomp(self, u1, n_var, out=None):
        u2 = self.xyplanes(n_var) if out is None else out
        self._check(load_library().sam_gpu_x2z_decomp(_p(u1), _p(u2), n_var, _p(u2)), "x2z_decomp")
        return u2

    def xy_trans_b(self, u1, n_var):
        u2 = self.phys(n_var)
        self._check(load_library().sam_gpu_xy_trans_b(_p(u1), _p(u2), n_var, None), "xy_trans_b")
        return u2

    def xy_trans_f(self, u1, n_var):
        u2 = self.wave(n_var)
        self._check(load_library().sam_gpu_xy_trans_f(_p(u1), _p(u2), n_var, None), "xy_trans_f")
        return u2

    def z2x_decomp(self, u1, n_var, out=None):
        u2 = u1 if out is None else out
        self._check(load_library().sam_gpu_z2x_decomp(_p(u1), _p(u2), n_var, None), "z2x_decomp")
        return u2

    def z_trans_f(self, u, n_var, isymm=None):
        iv = np.zeros(n_var, dtype=np.int32) if isymm is None else np.asarray(isymm, dtype=np.int32)
        self._check(load_library().sam_gpu_z_trans_f(_p(u), n_var, _p(iv), None, None), "z_trans_f")
        return u

    def vel_max(self, u):
        self._check(load_library().sam_gpu_vel_max(_p(u), None), "vel_max")
        return self.stats()

    def rhs(self, uu, u_sav=None):
        r = self.wave(self.lr)
        self._check(load_library().sam_gpu_rhs(_p(uu), _p(uu), _p(r), _p(u_sav), None), "rhs")
        return r

    def x_deriv(self, u):
        du = np.zeros_like(u, order="F")
        self._check(load_library().sam_gpu_x_deriv(_p(u), _p(du), None), "x_deriv")
        return du

    def y_deriv(self, u):
        du = np.zeros_like(u, order="F")
        self._check(load_library().sam_gpu_y_deriv(_p(u), _p(du), None), "y_deriv")
        return du

    # ---- subgrid models (haloed grids) and get_mean
    def filter(self, f_bar, n_var):
        f_hat = np.zeros((self.nx + 2, self.ny + 2, n_var), order="F")
        self._check(load_library().sam_gpu_filter(_p(f_bar), _p(f_hat), n_var), "filter")
        return f_hat

    def sm(self, u):
        vt = np.zeros((self.nx + 2, self.ny + 2, self.nz + 2), order="F")
        self._check(load_library().sam_gpu_sm(_p(u), None, None, _p(vt)), "sm")
        return vt

    def dm(self, u):
        vt = np.zeros((self.nx + 2, self.ny + 2, self.nz + 2), order="F")
        cds = np.zeros(1)
        self._check(load_library().sam_gpu_dm(_p(u), None, None, None, None, None, None, None, None, _p(vt),
                                              _p(cds)), "dm")
        return vt, float(cds[0])

    def get_mean(self, ufield, i_remove=0):
        """ufield: one field (Nze, Ny_min, Nx_min), modified in place when i_remove=1."""
        um = np.zeros(self.nze)
        jump = np.zeros(1)
        self._check(load_library().sam_gpu_get_mean(_p(ufield), 0, i_remove, _p(um), _p(jump), None), "get_mean")
        return um, float(jump[0])

    # ---- resident path
    def upload(self, u):
        self._check(load_library().sam_gpu_upload(_p(u)), "upload")

    def download(self, with_r=False, out=None):
        u = self.wave(self.lu) if out is None else out
        r = self.wave(self.lu + 1) if with_r else None
        self._check(load_library().sam_gpu_download(_p(u), _p(r)), "download")
        return (u, r) if with_r else u

    def stage(self, nrk):
        self._check(load_library().sam_gpu_stage(nrk), "stage")

    def step(self, nsteps=1):
        self._check(load_library().sam_gpu_step(nsteps), "step")

    def profile_stage(self, nrk, reps):
        """Mean ms of the five passes of stage nrk (CUDA events between them)."""
        ms = np.zeros(5, dtype=np.float32)
        self._check(load_library().sam_gpu_profile_stage(nrk, reps, ms.ctypes.data_as(C.c_void_p)), "profile")
        return dict(zip(("z_inv", "y_inv", "x_pass", "y_fwd", "z_fwd"), [float(x) for x in ms]))

    def autotune(self, reps=3):
        """Pick the fastest tiling and FFT schedule of each pass on the
        resident state; returns the choice."""
        self._check(load_library().sam_gpu_autotune(reps), "autotune")
        t = np.zeros(6, dtype=np.int32)
        self._check(load_library().sam_gpu_tiles(t.ctypes.data_as(C.c_void_p)), "tiles")
        out = dict(zip(TILE_KEYS, [int(x) for x in t]))
        out["fft_schedule"] = self.fft_schedule()
        return out

    def tiles(self):
        """The tiles in use (the autotuner's or set_tiles')."""
        t = np.zeros(6, dtype=np.int32)
        self._check(load_library().sam_gpu_tiles(t.ctypes.data_as(C.c_void_p)), "tiles")
        return dict(zip(TILE_KEYS, [int(x) for x in t]))

    def set_tiles(self, **tiles):
        """Set tiles by name (z_inv_rows, y_inv_cols, x_rows, x_group,
        y_fwd_planes, z_fwd_rows); the others keep their values."""
        cur = self.tiles()
        unknown = set(tiles) - set(TILE_KEYS)
        if unknown:
            raise ValueError(f"unknown tiles {sorted(unknown)}")
        cur.update(tiles)
        t = np.array([cur[k] for k in TILE_KEYS], dtype=np.int32)
        self._check(load_library().sam_gpu_set_tiles(t.ctypes.data_as(C.c_void_p)), "set_tiles")

    def set_fft_schedule(self, sched):
        """FFT schedule of the five passes (z inverse, y inverse, x, y forward,
        z forward) for length-256 lines: 0 the 16 x 16 register path, 1
        compile-time Stockham stages (8, 8, 4)."""
        a = np.ascontiguousarray(sched, dtype=np.int32)
        if a.shape != (5,):
            raise ValueError("set_fft_schedule: five values")
        self._check(load_library().sam_gpu_set_fft_schedule(a.ctypes.data_as(C.c_void_p)), "set_fft_schedule")

    def fft_schedule(self):
        a = np.zeros(5, dtype=np.int32)
        self._check(load_library().sam_gpu_fft_schedule(a.ctypes.data_as(C.c_void_p)), "fft_schedule")
        return [int(x) for x in a]

    def fp64_peak_tflops(self):
        t = C.c_double(0.0)
        self._check(load_library().sam_gpu_measure_fp64_peak(C.byref(t)), "measure_fp64_peak")
        return t.value

    # ---- diagnostics
    def spectra(self):
        lm = self.lm
        o = np.zeros(5 * lm + 3)
        self._check(load_library().sam_gpu_spectra(_p(o)), "spectra")
        return dict(ek=o[:lm], tk=o[lm:2 * lm], dk=o[2 * lm:3 * lm], vt=o[3 * lm:4 * lm],
                    sample=o[4 * lm:5 * lm], energy_w=o[5 * lm], div_rms=o[5 * lm + 1], div_max=o[5 * lm + 2])

    def set_forcing(self, seed, k_f=2.5, sigma=0.1, t_l=1.0):
        """Ornstein-Uhlenbeck forcing of 0 < |k| <= k_f applied after every
        step(); returns the number of forced modes (k_f <= 0 switches it off)."""
        n = C.c_int(0)
        self._check(load_library().sam_gpu_set_forcing(seed, k_f, sigma, t_l, C.byref(n)), "set_forcing")
        return n.value

    def set_les(self, model, c_smag=0.01, pr_t=1.0):
        """Subgrid closure coupled into every stage: 0 off, 1 Smagorinsky
        (C delta^2 = c_smag delta^2), 2 dynamic (dm.f's coefficient at stage
        1 of each step), 3 the learned closure (the network's per-point
        coefficients at stage 1 of each step); kappa_t = nu_t / pr_t
        (models 1, 2)."""
        self._check(load_library().sam_gpu_set_les(model, c_smag, pr_t), "set_les")

    def les_coef(self):
        """C delta^2 the closure last used."""
        v = C.c_double(0.0)
        self._check(load_library().sam_gpu_les_coef(C.byref(v)), "les_coef")
        return v.value

    # ---- learned closure
    @staticmethod
    def _f32(a, shape=None):
        a = np.ascontiguousarray(a, dtype=np.float32)
        if shape is not None:
            a = a.reshape(shape)
        return a

    def mlp_set(self, params):
        p = self._f32(params, (MLP_PARAMS,))
        self._check(load_library().sam_gpu_mlp_set(p.ctypes.data_as(C.c_void_p), MLP_PARAMS), "mlp_set")

    def mlp_get(self):
        p = np.zeros(MLP_PARAMS, dtype=np.float32)
        self._check(load_library().sam_gpu_mlp_get(p.ctypes.data_as(C.c_void_p), MLP_PARAMS), "mlp_get")
        return p

    def mlp_forward(self, features):
        f = self._f32(features).reshape(-1, MLP_FEATURES)
        out = np.zeros((len(f), 2), dtype=np.float32)
        self._check(load_library().sam_gpu_mlp_forward(f.ctypes.data_as(C.c_void_p), len(f),
                                                       out.ctypes.data_as(C.c_void_p)), "mlp_forward")
        return out

    def mlp_grad(self, features, target):
        f = self._f32(features).reshape(-1, MLP_FEATURES)
        t = self._f32(target).reshape(-1, 2)
        g = np.zeros(MLP_PARAMS, dtype=np.float32)
        loss = C.c_float(0.0)
        self._check(load_library().sam_gpu_mlp_grad(f.ctypes.data_as(C.c_void_p), t.ctypes.data_as(C.c_void_p),
                                                    len(f), g.ctypes.data_as(C.c_void_p), C.byref(loss)),
                    "mlp_grad")
        return g, loss.value

    def mlp_set_backward(self, tensor_cores=True):
        """Backward pass on the tensor cores (default) or on the CUDA cores."""
        self._check(load_library().sam_gpu_mlp_set_backward(1 if tensor_cores else 0), "mlp_set_backward")

    def mlp_train(self, features, target, steps, batch=8192, lr=1e-3):
        f = self._f32(features).reshape(-1, MLP_FEATURES)
        t = self._f32(target).reshape(-1, 2)
        hist = np.zeros(max(steps, 1), dtype=np.float32)
        self._check(load_library().sam_gpu_mlp_train(f.ctypes.data_as(C.c_void_p), t.ctypes.data_as(C.c_void_p),
                                                     len(f), steps, batch, lr, hist.ctypes.data_as(C.c_void_p)),
                    "mlp_train")
        return hist[:steps]

    def box_filter(self, f):
        """Block means over f^3 cells of u, [T], u_a u_b, [u_a T]: (X, Y, Z, Lu+Lr)."""
        n = self.cfg
        out = np.zeros((n.nx // f, n.ny // f, n.nz // f, self.lu + self.lr), order="F")
        self._check(load_library().sam_gpu_box_filter(f, _p(out)), "box_filter")
        return out

    def closure_inputs(self):
        """(features [Nx*Ny*Nz][12] float32 (BF16 values), grads (Nx,Ny,Nz,Lr+3))."""
        n = self.cfg
        npt = n.nx * n.ny * n.nz
        raw = np.zeros((npt, 16), dtype=np.uint16)
        grads = np.zeros((n.nx, n.ny, n.nz, self.lr + 3), order="F")
        self._check(load_library().sam_gpu_closure_inputs(raw.ctypes.data_as(C.c_void_p), _p(grads)),
                    "closure_inputs")
        feat = (raw[:, :12].astype(np.uint32) << 16).view(np.float32)
        return feat, grads

    def mma_selftest(self, a, b):
        a = self._f32(a, (128, 16))
        b = self._f32(b, (64, 16))
        d = np.zeros((128, 64), dtype=np.float32)
        self._check(load_library().sam_gpu_mma_selftest(a.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p),
                                                       d.ctypes.data_as(C.c_void_p)), "mma_selftest")
        return d

    def planes(self, k_xy=(), j_xz=(), i_yz=()):
        """Planes output of the resident state (sam.f:145-166, write_planes.f),
        1-based plane indices: xy (Nx,Ny,2Lu,n_xy), xz (Nx,Nz,2Lu,n_xz),
        yz (Ny,Nz,2Lu,n_yz) and the mean profiles (Nz,Lu)."""
        lu = self.lu
        ia = [np.ascontiguousarray(x, dtype=np.int32) for x in (k_xy, j_xz, i_yz)]
        xy = np.zeros((self.nx, self.ny, 2 * lu, len(ia[0])), order="F")
        xz = np.zeros((self.nx, self.nz, 2 * lu, len(ia[1])), order="F")
        yz = np.zeros((self.ny, self.nz, 2 * lu, len(ia[2])), order="F")
        mean = np.zeros((self.nz, lu), order="F")
        self._check(load_library().sam_gpu_planes(
            _p(ia[0]) if len(ia[0]) else None, len(ia[0]), _p(ia[1]) if len(ia[1]) else None, len(ia[1]),
            _p(ia[2]) if len(ia[2]) else None, len(ia[2]), _p(xy) if len(ia[0]) else None,
            _p(xz) if len(ia[1]) else None, _p(yz) if len(ia[2]) else None, _p(mean)), "planes")
        return dict(xy=xy, xz=xz, yz=yz, mean=mean)

    def div_check(self):
        o = np.zeros(4)
        self._check(load_library().sam_gpu_div_check(_p(o)), "div_check")
        return dict(div_avg=o[0], div_rms=o[1], div_max=o[2], n_div=o[3])

    def cl_energy(self):
        e = C.c_double(0.0)
        self._check(load_library().sam_gpu_cl_energy(C.byref(e)), "cl_energy")
        return e.value

    # ---- forcing and restart files
    def force(self, ek_0, k_force):
        self._check(load_library().sam_gpu_force(_p(np.ascontiguousarray(ek_0, dtype=np.float64)), k_force),
                    "force")

    def write_field(self, fname):
        self._check(load_library().sam_gpu_write_field(fname.encode()), "write_field")

    def read_field(self, fname):
        self._check(load_library().sam_gpu_read_field(fname.encode()), "read_field")

    def write_header(self, fname, nt):
        self._check(load_library().sam_gpu_write_header(fname.encode(), nt), "write_header")

    def read_header(self, fname):
        nt = C.c_int(0)
        self._check(load_library().sam_gpu_read_header(fname.encode(), C.byref(nt)), "read_header")
        return nt.value

    # ---- initial fields
    def init_taylor_green(self):
        self._check(load_library().sam_gpu_init_taylor_green(), "init_taylor_green")

    def init_random(self, seed, kind_u=6, flct_u=1.0, kind_t=6, flct_t=0.1):
        self._check(load_library().sam_gpu_init_random(seed, kind_u, flct_u, kind_t, flct_t), "init_random")

    def init_packet(self, seed, k0=(8, 0, 16), sigma=np.pi / 4, amplitude=0.05, noise=0.01):
        self._check(load_library().sam_gpu_init_packet(seed, k0[0], k0[1], k0[2], sigma, amplitude, noise),
                    "init_packet")


class _Member(SamGpu):
    """One member of a SamEnsemble: every SamGpu method, acting on the
    member (selected before each call through __getattribute__)."""

    def __init__(self, ens, index, cfg):
        self._ens, self._index, self.cfg = ens, index, cfg
        load_library().sam_gpu_ensemble_select(index)
        d = np.zeros(11, dtype=np.int32)
        self._check(load_library().sam_gpu_dims(d.ctypes.data_as(C.c_void_p)), "sam_gpu_dims")
        (self.nx_min, self.ny_min, self.nz_min, self.nze, self.lu, self.lr, self.kx_max, self.ky_max,
         self.kz_max, self.lm, self.nx2) = [int(x) for x in d]
        self.nx, self.ny, self.nz = cfg.nx, cfg.ny, cfg.nz

    def __getattribute__(self, name):
        attr = object.__getattribute__(self, name)
        if callable(attr) and not name.startswith("__") and name not in ("_check", "wave", "zblocks", "xyplanes",
                                                                          "phys"):
            self._check(load_library().sam_gpu_ensemble_select(object.__getattribute__(self, "_index")),
                        "ensemble_select")
        return attr

    def set_les(self, model, c_smag=0.01, pr_t=1.0):
        SamGpu.set_les(self, model, c_smag, pr_t)
        self._les = model

    def close(self):
        pass


def _persistent_eligible(cfg, les):
    """Whether a member runs in the ensemble's persistent launch (the C
    library's rule: FP32 bulk form, no closure, lengths with a compile-time
    FFT path)."""
    return cfg.precision == 32 and les == 0 and all(n in (32, 64, 96, 128) for n in (cfg.nx, cfg.ny, cfg.nz))


class SamEnsemble:
    """Independent runs advanced together (sam_gpu_ensemble_*): one CUDA graph
    per step over every member, each member its own branch and buffers."""

    def __init__(self, cfgs):
        lib = load_library()
        if SamGpu._live is not None:
            SamGpu._live.close()
        defaults = dict(n_dealias=1, i_strat=0, i_cfl=0, nrk_max=3, rot_sav=0, i_les=0, precision=64,
                        xl=2 * np.pi, yl=2 * np.pi, zl=2 * np.pi, vis=0.0, pr=1.0, dt0=0.01, cfl0=0.5,
                        buoy_fac_x=0.0, buoy_fac_z=0.0, lapse=0.0, cos_theta=1.0, sin_theta=0.0, c_smag=0.01)
        arr = (Config * len(cfgs))()
        for i, cfg in enumerate(cfgs):
            d = dict(defaults)
            d.update(cfg)
            for k, v in d.items():
                setattr(arr[i], k, v)
        self._arr = arr
        rc = lib.sam_gpu_ensemble_create(C.cast(arr, C.c_void_p), len(cfgs))
        if rc != SAM_GPU_OK:
            raise SamGpuError(f"ensemble_create failed ({ERRORS.get(rc, rc)}): "
                              + lib.sam_gpu_error_string().decode(errors="replace"))
        SamGpu._live = self
        self._persistent = 3
        self.members = [_Member(self, i, arr[i]) for i in range(len(cfgs))]

    def __len__(self):
        return len(self.members)

    def __getitem__(self, i):
        return self.members[i]

    def step(self, nsteps=1):
        rc = load_library().sam_gpu_ensemble_step(nsteps)
        if rc != SAM_GPU_OK:
            raise SamGpuError(f"ensemble_step failed ({ERRORS.get(rc, rc)}): "
                              + load_library().sam_gpu_error_string().decode(errors="replace"))

    def set_persistent(self, on=True, ctas_per_sm=3):
        """Members that qualify advance in one persistent launch per RK3 stage
        (on; at most ctas_per_sm CTAs per SM) or each in its own branch of the
        step graph (off)."""
        rc = load_library().sam_gpu_ensemble_set_persistent(ctas_per_sm if on else 0)
        if rc != SAM_GPU_OK:
            raise SamGpuError(f"ensemble_set_persistent failed ({ERRORS.get(rc, rc)})")
        self._persistent = ctas_per_sm if on else 0

    def autotune(self, reps=3, persistent_members=False):
        """The autotuner over the ensemble: for each class of members that run
        in branches of the step graph (grid, precision, closure model) one
        member is tuned on its resident state (sam_gpu_autotune) and its tiles
        and FFT schedules are copied to the others of the class
        (sam_gpu_set_tiles, sam_gpu_set_fft_schedule).  Members of the
        persistent launch keep the tiles the launch is sized for unless
        persistent_members is set (tiles tuned on a member's own kernels are
        larger than the persistent launch favours: 4479 -> 4391 member-steps/s
        on the 96-member benchmark ensemble).  Call after the members' set-up
        (closures), before stepping; returns the tiles per class."""
        done = {}
        for m in self.members:
            c, les = m.cfg, getattr(m, "_les", 0)
            if self._persistent and _persistent_eligible(c, les) and not persistent_members:
                continue
            key = (c.nx, c.ny, c.nz, c.precision, les)
            if key not in done:
                done[key] = m.autotune(reps)
            else:
                t = dict(done[key])
                sched = t.pop("fft_schedule")
                m.set_tiles(**t)
                m.set_fft_schedule(sched)
        return done

    def persistent_members(self):
        n = C.c_int(0)
        rc = load_library().sam_gpu_ensemble_persistent_members(C.byref(n))
        if rc != SAM_GPU_OK:
            raise SamGpuError(f"ensemble_persistent_members failed ({ERRORS.get(rc, rc)})")
        return n.value

    def close(self):
        if SamGpu._live is self:
            load_library().sam_gpu_ensemble_destroy()
            SamGpu._live = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
