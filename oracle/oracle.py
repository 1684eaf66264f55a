"""ctypes access to the CPU oracle -- TEST INFRASTRUCTURE ONLY.

The oracle is a plain-C FP64 restatement of the SAM hot path (sam_oracle.c).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the checker (or the timed CPU baseline); the shipped
CUDA library never calls it.

Arrays follow the reference layouts in Fortran order:
  wave space   complex128 (Nze, Ny_min, Nx_min, n)   sam.f:93
  z_trans_b    complex128 (Ny_min, Nx_min, Nze, n)   z_trans_b.f:10-13
  x2z output   complex128 (Ny, Nx/2, Nz, n)          x2z_decomp.f:17
  physical     float64    (Nx, Ny, Nz, n)            sam.f:94
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
SOURCES = ["sam_oracle.c", "so_fft.c"]


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (OpenMP, -O3, portable flags)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    hdrs = [os.path.join(HERE, h) for h in ("sam_oracle.h", "so_fft.h")]
    if not force and os.path.exists(LIB_PATH):
        t = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(s) <= t for s in srcs + hdrs):
            return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O3", "-std=c11", "-fopenmp", "-fPIC", "-shared", "-o", tmp, *srcs, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class SoConfig(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("n_dealias", C.c_int), ("i_strat", C.c_int), ("i_cfl", C.c_int),
        ("nrk_max", C.c_int), ("rot_sav", C.c_int), ("i_les", C.c_int),
        ("nthreads", C.c_int),
        ("xl", C.c_double), ("yl", C.c_double), ("zl", C.c_double),
        ("vis", C.c_double), ("pr", C.c_double),
        ("dt0", C.c_double), ("cfl0", C.c_double),
        ("buoy_fac_x", C.c_double), ("buoy_fac_z", C.c_double), ("lapse", C.c_double),
        ("cos_theta", C.c_double), ("sin_theta", C.c_double),
        ("c_smag", C.c_double),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        P = C.c_void_p
        _lib.so_create.restype = P
        _lib.so_create.argtypes = [C.POINTER(SoConfig)]
        _lib.so_destroy.argtypes = [P]
        _lib.so_dims.argtypes = [P, P]
        _lib.so_set_time.argtypes = [P, C.c_double, C.c_double]
        _lib.so_stats.argtypes = [P, P]
        for name in ("so_z_trans_b", "so_x2z_decomp", "so_xy_trans_b", "so_xy_trans_f", "so_z2x_decomp"):
            getattr(_lib, name).argtypes = [P, P, P, C.c_int]
        _lib.so_z_trans_f.argtypes = [P, P, C.c_int]
        _lib.so_vel_max.argtypes = [P, P]
        _lib.so_rhs.argtypes = [P, P, P, P, C.c_int]
        _lib.so_stage.argtypes = [P, P, P, C.c_int]
        _lib.so_steps.argtypes = [P, P, P, C.c_int]
        _lib.so_spectra.argtypes = [P, P, P, P]
        _lib.so_div_check.argtypes = [P, P, P]
        _lib.so_cl_energy.argtypes = [P, P]
        _lib.so_cl_energy.restype = C.c_double
        _lib.so_get_mean.argtypes = [P, P, C.c_int, P]
        _lib.so_get_mean.restype = C.c_double
        _lib.so_x_deriv.argtypes = [P, P, P]
        _lib.so_y_deriv.argtypes = [P, P, P]
        _lib.so_filter.argtypes = [P, P, P, C.c_int]
        _lib.so_sm.argtypes = [P, P, P]
        _lib.so_dm.argtypes = [P, P, P]
        _lib.so_dm.restype = C.c_double
        _lib.so_init_taylor_green.argtypes = [P, P]
        _lib.so_init_random.argtypes = [P, P, C.c_ulonglong, C.c_int, C.c_double, C.c_int, C.c_double]
        _lib.so_init_gw_plane.argtypes = [P, P] + [C.c_double] * 8
        _lib.so_init_packet.argtypes = [P, P, C.c_ulonglong, C.c_int, C.c_int, C.c_int,
                                        C.c_double, C.c_double, C.c_double]
        _lib.so_fft_line.argtypes = [C.c_int, C.c_int, P]
        _lib.so_force.argtypes = [P, P, P, C.c_int]
        _lib.so_set_forcing.argtypes = [P, C.c_ulonglong, C.c_double, C.c_double, C.c_double]
        _lib.so_set_les.argtypes = [P, C.c_int, C.c_double, C.c_double]
        _lib.so_les_coef.argtypes = [P]
        _lib.so_les_coef.restype = C.c_double
        _lib.so_mlp_set.argtypes = [P, P]
        _lib.so_closure_invariants.argtypes = [P, P, P, C.c_double, C.c_double, C.c_double, C.c_double, P]
        _lib.so_planes.argtypes = [P, P, P, P, C.c_int, P, C.c_int, P, C.c_int, P, P, P, P]
        _lib.so_write_field.argtypes = [P, C.c_char_p, P]
        _lib.so_read_field.argtypes = [P, C.c_char_p, P]
    return _lib


def fft_line(data: np.ndarray, kind: str) -> np.ndarray:
    """One FFTPACK-convention transform: 'cfftf', 'cfftb' (complex input) or
    'rfftf', 'rfftb' (real input in FFTPACK's packed layout)."""
    k = {"cfftf": 0, "cfftb": 1, "rfftf": 2, "rfftb": 3}[kind]
    a = np.array(data, dtype=np.complex128 if k <= 1 else np.float64, copy=True)
    rc = lib().so_fft_line(len(a), k, a.ctypes.data_as(C.c_void_p))
    if rc:
        raise ValueError(f"unsupported length {len(a)}")
    return a


def closure_invariants(S, g, w, bz=0.0, n2=0.0, dsq=1.0, nu=1.0):
    """The learned closure's 12 inputs of one point (oracle formulas)."""
    S = np.ascontiguousarray(S, dtype=np.float64)
    g = np.ascontiguousarray(g, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    f = np.zeros(12, dtype=np.float32)
    v = C.c_void_p
    lib().so_closure_invariants(S.ctypes.data_as(v), g.ctypes.data_as(v), w.ctypes.data_as(v), bz, n2, dsq, nu,
                                f.ctypes.data_as(v))
    return f


def _p(a: np.ndarray):
    assert a.flags["F_CONTIGUOUS"] or a.ndim <= 1, "arrays must be Fortran-ordered"
    return a.ctypes.data_as(C.c_void_p)


@dataclass
class Dims:
    nx: int
    ny: int
    nz: int
    nx_min: int
    ny_min: int
    nz_min: int
    nze: int
    lu: int
    lr: int
    kx_max: int
    ky_max: int
    kz_max: int
    lm: int
    nx2: int


class Oracle:
    """One oracle context: the reference's COMMON state for one run."""

    def __init__(self, **cfg):
        self.cfg = SoConfig()
        defaults = dict(n_dealias=1, i_strat=0, i_cfl=0, nrk_max=3, rot_sav=0, i_les=0, nthreads=0,
                        xl=2 * np.pi, yl=2 * np.pi, zl=2 * np.pi, vis=0.0, pr=1.0, dt0=0.01, cfl0=0.5,
                        buoy_fac_x=0.0, buoy_fac_z=0.0, lapse=0.0, cos_theta=1.0, sin_theta=0.0,
                        c_smag=0.01)
        defaults.update(cfg)
        for k, v in defaults.items():
            setattr(self.cfg, k, v)
        self.h = lib().so_create(C.byref(self.cfg))
        if not self.h:
            raise ValueError(f"oracle rejected config {cfg}")
        d = np.zeros(11, dtype=np.int32)
        lib().so_dims(self.h, d.ctypes.data_as(C.c_void_p))
        self.d = Dims(self.cfg.nx, self.cfg.ny, self.cfg.nz, *[int(x) for x in d[:3]], int(d[3]),
                      *[int(x) for x in d[4:11]])

    def close(self):
        if self.h:
            lib().so_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- arrays in the reference layouts
    def wave(self, n):
        d = self.d
        return np.zeros((d.nze, d.ny_min, d.nx_min, n), dtype=np.complex128, order="F")

    def zblocks(self, n):
        d = self.d
        return np.zeros((d.ny_min, d.nx_min, d.nze, n), dtype=np.complex128, order="F")

    def xyplanes(self, n):
        d = self.d
        return np.zeros((d.ny, d.nx2, d.nz, n), dtype=np.complex128, order="F")

    def phys(self, n):
        d = self.d
        return np.zeros((d.nx, d.ny, d.nz, n), dtype=np.float64, order="F")

    # ---- state
    def set_time(self, time, dt):
        lib().so_set_time(self.h, time, dt)

    def stats(self):
        o = np.zeros(18)
        lib().so_stats(self.h, _p(o))
        return dict(time=o[0], dt=o[1], u_avg=o[2:6].copy(), u_var=o[6:10].copy(), u_max=o[10:14].copy(),
                    energy=o[14], cfl_x=o[15], cfl_y=o[16], cfl_z=o[17])

    # ---- transforms
    def z_trans_b(self, u1, n_var):
        u2 = self.zblocks(n_var)
        lib().so_z_trans_b(self.h, _p(u1), _p(u2), n_var)
        return u2

    def x2z_decomp(self, u1, n_var, out=None):
        u2 = self.xyplanes(n_var) if out is None else out
        lib().so_x2z_decomp(self.h, _p(u1), _p(u2), n_var)
        return u2

    def xy_trans_b(self, u1, n_var):
        """Returns the physical fields; u1 is overwritten as in the reference."""
        u2 = self.phys(n_var)
        lib().so_xy_trans_b(self.h, _p(u1), _p(u2), n_var)
        return u2

    def xy_trans_f(self, u1, n_var):
        """u1 (physical) is overwritten with its x transforms, as in the reference."""
        u2 = self.wave(n_var)
        lib().so_xy_trans_f(self.h, _p(u1), _p(u2), n_var)
        return u2

    def z_trans_f(self, u, n_var):
        lib().so_z_trans_f(self.h, _p(u), n_var)
        return u

    # ---- physics
    def vel_max(self, u):
        lib().so_vel_max(self.h, _p(u))
        return self.stats()

    def rhs(self, uu, u_sav, nrk):
        """uu (Nx,Ny,Nz,Lr) with the physical fields first; returns r (Lr fields)."""
        r = self.wave(self.d.lr)
        lib().so_rhs(self.h, _p(uu), _p(r), _p(u_sav) if u_sav is not None else None, nrk)
        return r

    def stage(self, u, r, nrk):
        lib().so_stage(self.h, _p(u), _p(r), nrk)

    def steps(self, u, r, n):
        lib().so_steps(self.h, _p(u), _p(r), n)

    # ---- diagnostics
    def spectra(self, u, r):
        lm = self.d.lm
        o = np.zeros(5 * lm + 3)
        lib().so_spectra(self.h, _p(u), _p(r), _p(o))
        return dict(ek=o[:lm], tk=o[lm:2 * lm], dk=o[2 * lm:3 * lm], vt=o[3 * lm:4 * lm],
                    sample=o[4 * lm:5 * lm], energy_w=o[5 * lm], div_rms=o[5 * lm + 1], div_max=o[5 * lm + 2])

    def div_check(self, u):
        o = np.zeros(4)
        lib().so_div_check(self.h, _p(u), _p(o))
        return dict(div_avg=o[0], div_rms=o[1], div_max=o[2], n_div=o[3])

    def cl_energy(self, u):
        return lib().so_cl_energy(self.h, _p(u))

    def get_mean(self, ufield, i_remove=0):
        um = np.zeros(self.d.nze)
        jump = lib().so_get_mean(self.h, _p(ufield), i_remove, _p(um))
        return um, jump

    def x_deriv(self, u):
        du = np.zeros_like(u, order="F")
        lib().so_x_deriv(self.h, _p(u), _p(du))
        return du

    def y_deriv(self, u):
        du = np.zeros_like(u, order="F")
        lib().so_y_deriv(self.h, _p(u), _p(du))
        return du

    def set_forcing(self, seed, k_f=2.5, sigma=0.1, t_l=1.0):
        n = lib().so_set_forcing(self.h, seed, k_f, sigma, t_l)
        if n < 0:
            raise ValueError("too many forced modes")
        return n

    def set_les(self, model, c_smag=0.01, pr_t=1.0):
        """Subgrid closure coupled into stage(): 0 off, 1 Smagorinsky,
        2 dynamic (dm.f coefficient at nrk = 1); kappa_t = nu_t / pr_t."""
        if lib().so_set_les(self.h, model, c_smag, pr_t):
            raise ValueError("bad LES arguments")

    def mlp_set(self, params):
        """Parameters of the learned closure (model 3 of set_les)."""
        p = np.ascontiguousarray(params, dtype=np.float32)
        assert p.size == 5122
        lib().so_mlp_set(self.h, p.ctypes.data_as(C.c_void_p))

    def les_coef(self):
        """C delta^2 last used by the coupled closure."""
        return lib().so_les_coef(self.h)

    def planes(self, u, p, k_xy=(), j_xz=(), i_yz=()):
        """Planes output of sam.f:145-166 / write_planes.f (1-based plane
        indices): xy (Nx,Ny,2Lu,n_xy), xz (Nx,Nz,2Lu,n_xz), yz (Ny,Nz,2Lu,n_yz),
        mean (Nz,Lu); p is the pressure field r(Lu+1) in wave space."""
        d = self.d
        n_out = 2 * d.lu
        ia = [np.ascontiguousarray(x, dtype=np.int32) for x in (k_xy, j_xz, i_yz)]
        xy = np.zeros((d.nx, d.ny, n_out, max(len(ia[0]), 1)), order="F")
        xz = np.zeros((d.nx, d.nz, n_out, max(len(ia[1]), 1)), order="F")
        yz = np.zeros((d.ny, d.nz, n_out, max(len(ia[2]), 1)), order="F")
        mean = np.zeros((d.nz, d.lu), order="F")
        u = np.asfortranarray(u)
        p = np.asfortranarray(p)
        rc = lib().so_planes(self.h, _p(u), _p(p), _p(ia[0]), len(ia[0]), _p(ia[1]), len(ia[1]), _p(ia[2]),
                             len(ia[2]), _p(xy), _p(xz), _p(yz), _p(mean))
        if rc:
            raise ValueError("so_planes: plane index out of range")
        return dict(xy=xy[..., :len(ia[0])], xz=xz[..., :len(ia[1])], yz=yz[..., :len(ia[2])], mean=mean)

    def filter(self, f_bar, n_var):
        d = self.d
        f_hat = np.zeros((d.nx + 2, d.ny + 2, n_var), order="F")
        lib().so_filter(self.h, _p(f_bar), _p(f_hat), n_var)
        return f_hat

    def sm(self, u):
        d = self.d
        vt = np.zeros((d.nx + 2, d.ny + 2, d.nz + 2), order="F")
        lib().so_sm(self.h, _p(u), _p(vt))
        return vt

    def dm(self, u):
        d = self.d
        vt = np.zeros((d.nx + 2, d.ny + 2, d.nz + 2), order="F")
        cds = lib().so_dm(self.h, _p(u), _p(vt))
        return vt, cds

    # ---- forcing and restart files
    def force(self, u, ek_0, k_force):
        lib().so_force(self.h, _p(u), _p(np.ascontiguousarray(ek_0, dtype=np.float64)), k_force)
        return u

    def write_field(self, fname, u):
        assert lib().so_write_field(self.h, fname.encode(), _p(u)) == 0

    def read_field(self, fname):
        u = self.wave(self.d.lu)
        rc = lib().so_read_field(self.h, fname.encode(), _p(u))
        return u if rc == 0 else rc

    # ---- initial fields
    def init_taylor_green(self):
        u = self.wave(self.d.lu)
        rc = lib().so_init_taylor_green(self.h, _p(u))
        assert rc == 0
        return u

    def init_random(self, seed, kind_u=6, flct_u=1.0, kind_t=6, flct_t=0.1):
        u = self.wave(self.d.lu)
        lib().so_init_random(self.h, _p(u), seed, kind_u, flct_u, kind_t, flct_t)
        return u

    def init_gw_plane(self, amplitude, lambda_x, lambda_z, omega_i, k_w, m_w, lapse0, uo=0.0):
        u = self.wave(self.d.lu)
        rc = lib().so_init_gw_plane(self.h, _p(u), amplitude, lambda_x, lambda_z, omega_i, k_w, m_w, lapse0, uo)
        assert rc == 0
        return u

    def init_packet(self, seed, k0=(8, 0, 16), sigma=np.pi / 4, amplitude=0.05, noise=0.01):
        u = self.wave(self.d.lu)
        lib().so_init_packet(self.h, _p(u), seed, k0[0], k0[1], k0[2], sigma, amplitude, noise)
        return u
