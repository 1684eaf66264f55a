"""Parity of the CUDA path (through the C ABI) with the oracle.

FP64 bar: per-routine results within 1e-13 of the oracle relative to the
field's largest magnitude; full RK3 runs within 1e-12 per field after N steps
(the FFT factorisations differ from the oracle's, so agreement is to
rounding, not bitwise).
"""
import json
import os

import numpy as np
import pytest

import oracle as O
from sam_gb300 import SamGpu

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "kats.json")))
TOL_ROUTINE = 1e-13
TOL_RUN = 1e-12

GRIDS = [
    dict(nx=16, ny=16, nz=16, i_strat=1),
    dict(nx=24, ny=32, nz=36, i_strat=1, xl=3.0, yl=2.0, zl=1.5),
    dict(nx=72, ny=1, nz=24, i_strat=1, xl=3.0, yl=0.05, zl=1.0),
    dict(nx=32, ny=32, nz=32, i_strat=0),
    dict(nx=48, ny=20, nz=96, i_strat=1),
    # length-256 lines take the 16 x 16 register path: x and y, then z
    dict(nx=256, ny=256, nz=12, i_strat=1),
    dict(nx=16, ny=20, nz=256, i_strat=1),
    # compile-time radix paths (128, 64, 512, 96; 96 in z above) and the
    # longest line (1024)
    dict(nx=128, ny=64, nz=128, i_strat=1),
    dict(nx=512, ny=6, nz=10, i_strat=0),
    dict(nx=12, ny=10, nz=512, i_strat=1),
    dict(nx=1024, ny=2, nz=6, i_strat=1),
    dict(nx=96, ny=96, nz=8, i_strat=1),
]


def relerr(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def pair(**kw):
    base = dict(vis=1e-2, pr=0.7, dt0=0.01, buoy_fac_z=1.0 if kw.get("i_strat") else 0.0,
                lapse=1.0 if kw.get("i_strat") else 0.0)
    base.update(kw)
    return SamGpu(**base), O.Oracle(**base)


@pytest.mark.parametrize("grid", GRIDS)
def test_backward_transforms(gpu_lib, grid):
    g, o = pair(**grid)
    d = o.d
    u = o.init_random(17)
    zb_o = o.z_trans_b(u, d.lu)
    zb_g = g.z_trans_b(u, d.lu)
    assert relerr(zb_g, zb_o) < TOL_ROUTINE
    # x2z: columns kx >= Nx_min must be left untouched
    sentinel = np.full((d.ny, d.nx2, d.nz, d.lu), 7.0 + 3.0j, order="F")
    xy_g = g.x2z_decomp(zb_o, d.lu, out=sentinel.copy(order="F"))
    xy_o = o.x2z_decomp(zb_o, d.lu, out=sentinel.copy(order="F"))
    assert np.array_equal(xy_g, xy_o)
    ph_o = o.xy_trans_b(xy_o.copy(order="F"), d.lu)
    ph_g = g.xy_trans_b(xy_o.copy(order="F"), d.lu)
    assert relerr(ph_g, ph_o) < TOL_ROUTINE


@pytest.mark.parametrize("grid", GRIDS)
def test_forward_transforms(gpu_lib, grid):
    g, o = pair(**grid)
    d = o.d
    rng = np.random.default_rng(3)
    ph = np.asfortranarray(rng.standard_normal((d.nx, d.ny, d.nz, d.lu)))
    w_o = o.xy_trans_f(ph.copy(order="F"), d.lu)
    w_g = g.xy_trans_f(ph.copy(order="F"), d.lu)
    assert relerr(w_g, w_o) < TOL_ROUTINE
    # z2x with one rank is the identity
    assert np.array_equal(g.z2x_decomp(w_g.copy(order="F"), d.lu), w_g)
    zo = o.z_trans_f(w_o.copy(order="F"), d.lu)
    zg = g.z_trans_f(w_o.copy(order="F"), d.lu)
    assert relerr(zg[: d.nz_min], zo[: d.nz_min]) < TOL_ROUTINE


@pytest.mark.parametrize("grid", GRIDS[:4] + GRIDS[5:])
@pytest.mark.parametrize("nrk", [1, 2])
def test_rhs_and_vel_max(gpu_lib, grid, nrk):
    g, o = pair(i_cfl=1, cfl0=0.5, **grid)
    d = o.d
    u = o.init_random(29)
    ph = o.xy_trans_b(o.x2z_decomp(o.z_trans_b(u, d.lu), d.lu), d.lu)
    uu = o.phys(d.lr)
    uu[..., : d.lu] = ph
    usav = None
    if d.lu == 4:
        usav = np.asfortranarray(u[: d.nz_min, :, :, 2:4])
    o.set_time(0.0, 0.01)
    g.set_tstep(nrk, 0.01, 0.0)
    r_o = o.rhs(uu.copy(order="F"), usav, nrk)
    r_g = g.rhs(uu.copy(order="F"), usav)
    for n in range(d.lu + 1):
        assert relerr(r_g[: d.nz_min, :, :, n], r_o[: d.nz_min, :, :, n]) < TOL_ROUTINE, n
    so, sg = o.stats(), g.stats()
    if nrk == 1:
        np.testing.assert_allclose(sg["u_max"][: d.lu], so["u_max"][: d.lu], rtol=0, atol=0)
        np.testing.assert_allclose(sg["u_var"][: d.lu], so["u_var"][: d.lu], rtol=1e-12)
        assert sg["dt"] == so["dt"]
        np.testing.assert_allclose([sg["cfl_x"], sg["cfl_y"], sg["cfl_z"]], [so["cfl_x"], so["cfl_y"], so["cfl_z"]],
                                   rtol=1e-15)


@pytest.mark.parametrize("grid", GRIDS)
def test_resident_stages(gpu_lib, grid):
    g, o = pair(**grid)
    d = o.d
    u = o.init_random(41)
    g.upload(u)
    r = o.wave(d.lr)
    for nrk in (1, 2, 3):
        o.stage(u, r, nrk)
        g.stage(nrk)
        ug, rg = g.download(with_r=True)
        for n in range(d.lu):
            assert relerr(ug[: d.nz_min, ..., n], u[: d.nz_min, ..., n]) < TOL_ROUTINE, (nrk, n)
            assert relerr(rg[: d.nz_min, ..., n], r[: d.nz_min, ..., n]) < TOL_ROUTINE, (nrk, n)
        assert relerr(rg[: d.nz_min, ..., d.lu], r[: d.nz_min, ..., d.lu]) < TOL_ROUTINE


# the grids with length-256 lines, run with the other FFT schedule of every
# pass (compile-time Stockham 8, 8, 4 instead of the 16 x 16 register path)
@pytest.mark.parametrize("grid", [g for g in GRIDS if 256 in (g["nx"], g["ny"], g["nz"])])
def test_resident_stages_stockham_schedule(gpu_lib, grid):
    g, o = pair(**grid)
    d = o.d
    g.set_fft_schedule([1, 1, 1, 1, 1])
    assert g.fft_schedule() == [1, 1, 1, 1, 1]
    u = o.init_random(43)
    g.upload(u)
    r = o.wave(d.lr)
    for nrk in (1, 2, 3):
        o.stage(u, r, nrk)
        g.stage(nrk)
        ug, rg = g.download(with_r=True)
        for n in range(d.lu):
            assert relerr(ug[: d.nz_min, ..., n], u[: d.nz_min, ..., n]) < TOL_ROUTINE, (nrk, n)
            assert relerr(rg[: d.nz_min, ..., n], r[: d.nz_min, ..., n]) < TOL_ROUTINE, (nrk, n)


def test_fft_schedules_agree_in_fp32(gpu_lib):
    """FP32 bulk form, 256 x 256 x 12: one step with each schedule (FP32
    round-off apart) and the rejection of an unknown schedule."""
    cfg = dict(nx=256, ny=256, nz=12, i_strat=1, vis=1e-2, dt0=0.01, buoy_fac_z=1.0, lapse=1.0)
    o = O.Oracle(**cfg)
    u = o.init_random(5)
    out = []
    for sched in ([0, 0, 0, 0, 0], [1, 1, 1, 1, 1]):
        g = SamGpu(precision=32, **cfg)
        g.set_fft_schedule(sched)
        g.upload(u)
        g.step(1)
        out.append(g.download())
        if sched[0] == 1:
            with pytest.raises(Exception):
                g.set_fft_schedule([2, 0, 0, 0, 0])
            assert g.fft_schedule() == [1, 1, 1, 1, 1]
        g.close()
    assert relerr(out[1], out[0]) < 1e-5


@pytest.mark.parametrize("case", [
    dict(ny=256, nz=12, i_strat=1, n_dealias=1),   # the benchmark's lines, stratified
    dict(ny=243, nz=10, i_strat=0, n_dealias=1),   # odd Ny: ragged tiles, unaligned pair stores
    dict(ny=40, nz=8, i_strat=1, n_dealias=0),     # no truncation: kx_max = 127
    dict(ny=36, nz=9, i_strat=1, n_dealias=2),
])
@pytest.mark.parametrize("x_rows", [2, 4, 8, 16])
def test_fused_fp32_x_pass_bit_identical(gpu_lib, case, x_rows):
    """The fused FP32 x pass at Nx = 256 (schedule 0) against the 16 x 16 path
    of the general kernel (schedule 2): two CFL steps, bit for bit, with
    vel_max's max |u| taken in the fused kernel at stage 1, for every x-pass
    tile height (1 to 8 row pairs: fewer lines than teams, more, ragged)."""
    cfg = dict(nx=256, i_cfl=1, cfl0=0.5, vis=2e-3, pr=1.0, buoy_fac_z=1.0, lapse=1.0, **case)
    o = O.Oracle(**cfg)
    u = o.init_random(11, 6, 1.0, 6, 0.1)
    o.close()
    out = []
    for sched in ([0, 0, 0, 0, 0], [0, 0, 2, 0, 0]):
        g = SamGpu(precision=32, **cfg)
        g.set_fft_schedule(sched)
        assert g.fft_schedule() == sched
        g.set_tiles(x_rows=x_rows)
        assert g.tiles()["x_rows"] == x_rows
        g.upload(u)
        g.step(2)
        out.append((g.download(), g.stats()["dt"]))
        g.close()
    (u0, dt0), (u2, dt2) = out
    assert np.isfinite(u0).all()
    assert dt0 == dt2
    assert np.array_equal(u0, u2), np.abs(u0 - u2).max() / np.abs(u2).max()


def test_taylor_green_64_200_steps(gpu_lib):
    """Config 1: Taylor-Green 64^3, nu = 1/400, dt = 0.01, 200 RK3 steps."""
    cfg = dict(nx=64, ny=64, nz=64, vis=1.0 / 400, dt0=0.01)
    g, o = SamGpu(**cfg), O.Oracle(**cfg)
    u = o.init_taylor_green()
    g.init_taylor_green()
    assert np.array_equal(g.download(), u)
    r = o.wave(o.d.lr)
    o.steps(u, r, 200)
    g.step(200)
    ug = g.download()
    for n in range(3):
        err = relerr(ug[: o.d.nz_min, ..., n], u[: o.d.nz_min, ..., n]) if n < 2 else \
            np.abs(ug[..., n] - u[..., n]).max() / np.abs(u[..., :2]).max()
        assert err < TOL_RUN, (n, err)
    assert abs(g.stats()["time"] - 2.0) < 1e-12


def test_stratified_cfl_run(gpu_lib):
    """Stratified k^4 exp(-2(k/4)^2) turbulence with CFL-chosen dt (config 2 at 32^3)."""
    cfg = dict(nx=32, ny=32, nz=32, i_strat=1, i_cfl=1, cfl0=0.5, vis=1.0 / 800, pr=1.0, buoy_fac_z=1.0,
               lapse=1.0)
    g, o = SamGpu(**cfg), O.Oracle(**cfg)
    u = o.init_random(0, 6, 1.0, 6, 0.1)
    g.init_random(0, 6, 1.0, 6, 0.1)
    assert relerr(g.download(), u) < 1e-14
    g.upload(u)
    r = o.wave(o.d.lr)
    o.steps(u, r, 20)
    g.step(20)
    ug = g.download()
    for n in range(4):
        assert relerr(ug[: o.d.nz_min, ..., n], u[: o.d.nz_min, ..., n]) < TOL_RUN, n
    so, sg = o.stats(), g.stats()
    assert abs(sg["dt"] - so["dt"]) <= 1e-13 * so["dt"]
    assert abs(sg["time"] - so["time"]) <= 1e-12


def test_gravity_wave_input_dat(gpu_lib):
    """The reference's input.dat case on the GPU against the exact RK3 solution."""
    gd = GOLD["gw_input_dat"]
    cfg = dict(nx=gd["nx"], ny=gd["ny"], nz=gd["nz"], xl=gd["xl"], yl=gd["yl"], zl=gd["zl"], i_strat=1,
               vis=gd["vis"], dt0=gd["dt"], buoy_fac_z=gd["grav"] / gd["to"], lapse=gd["lapse0"])
    g, o = SamGpu(**cfg), O.Oracle(**cfg)
    u0 = o.init_gw_plane(gd["amplitude"], gd["lambda_x"], gd["lambda_z"], gd["omega_i"], gd["k_w"], gd["m_w"],
                         gd["lapse0"], gd["uo"])
    g.upload(u0)
    g.step(gd["n_steps"])
    ug = g.download()
    amp = complex(gd["rk3_amplification_re"], gd["rk3_amplification_im"])
    assert np.abs(ug - u0 * amp).max() / np.abs(u0).max() < 1e-13


def test_initial_fields_match(gpu_lib):
    cfg = dict(nx=48, ny=32, nz=40, i_strat=1, buoy_fac_z=4.0, lapse=1.0)
    g, o = SamGpu(**cfg), O.Oracle(**cfg)
    g.init_random(123, 6, 1.0, 6, 0.1)
    assert relerr(g.download(), o.init_random(123, 6, 1.0, 6, 0.1)) < 1e-14
    g.init_packet(7, (8, 0, 16), np.pi / 4, 0.05, 0.01)
    up = o.init_packet(7, (8, 0, 16), np.pi / 4, 0.05, 0.01)
    assert relerr(g.download(), up) < 1e-13


def test_diagnostics(gpu_lib):
    cfg = dict(nx=32, ny=24, nz=40, i_strat=1, i_les=1, vis=1e-3, buoy_fac_z=1.0, lapse=1.0)
    g, o = SamGpu(**cfg), O.Oracle(**cfg)
    u = o.init_random(5)
    g.upload(u)
    r = o.wave(o.d.lr)
    o.stage(u, r, 1)
    g.stage(1)
    so = o.spectra(u, r)
    sg = g.spectra()
    for key in ("ek", "tk", "dk", "vt", "sample"):
        np.testing.assert_allclose(sg[key], so[key], rtol=1e-11, atol=1e-15 * np.abs(so[key]).max())
    assert abs(sg["energy_w"] - so["energy_w"]) < 1e-13 * so["energy_w"]
    assert sg["div_max"] < 1e-12 and so["div_max"] < 1e-12
    dg, do = g.div_check(), o.div_check(u)
    assert dg["div_max"] < 1e-12 and do["div_max"] < 1e-12
    assert abs(g.cl_energy() - o.cl_energy(u)) <= 1e-12 * o.cl_energy(u)


@pytest.mark.parametrize("dims", [(16, 12), (72, 1), (64, 48), (96, 30)])
def test_plane_derivatives(gpu_lib, dims):
    nx, ny = dims
    g, o = SamGpu(nx=nx, ny=ny, nz=8), O.Oracle(nx=nx, ny=ny, nz=8)
    f = np.asfortranarray(np.random.default_rng(1).standard_normal((nx, ny)))
    assert relerr(g.x_deriv(f), o.x_deriv(f)) < TOL_ROUTINE
    if ny > 1:
        assert relerr(g.y_deriv(f), o.y_deriv(f)) < TOL_ROUTINE


def test_fp32_bulk_error_bounded(gpu_lib):
    """Precision form (1): FP32 transforms, FP64 reductions; the error against
    the FP64 oracle is reported and bounded."""
    cfg = dict(nx=32, ny=32, nz=32, i_strat=1, vis=1.0 / 800, buoy_fac_z=1.0, lapse=1.0, dt0=0.005)
    g, o = SamGpu(precision=32, **cfg), O.Oracle(**cfg)
    u = o.init_random(2)
    g.upload(u)
    r = o.wave(o.d.lr)
    o.steps(u, r, 10)
    g.step(10)
    ug = g.download()
    for n in range(4):
        assert relerr(ug[: o.d.nz_min, ..., n], u[: o.d.nz_min, ..., n]) < 1e-5, n


def test_full_size_properties(gpu_lib):
    """256^3 stratified (the benchmark grid): size-independent checks -- the
    projected field stays solenoidal to round-off and one stage agrees with a
    second, independent upload of the same state."""
    cfg = dict(nx=256, ny=256, nz=256, i_strat=1, vis=1e-4, buoy_fac_z=4.0, lapse=1.0, dt0=1e-3)
    g = SamGpu(**cfg)
    g.init_packet(1, (8, 0, 16), np.pi / 4, 0.05, 0.01)
    u0 = g.download()
    g.step(2)
    dc = g.div_check()
    assert dc["div_max"] < 1e-11
    u1 = g.download()
    g.upload(u0)
    g.step(2)
    assert np.array_equal(g.download(), u1)  # deterministic replay
    st = g.stats()
    assert st["nonfinite"] == 0 and np.isfinite(st["energy"])


def test_fp32_vel_max_sums_from_wave_space(gpu_lib):
    """The FP32 form takes vel_max's sums from the state in wave space
    (Parseval, FP64 arithmetic) and max |u| from the physical field: after
    one step its statistics agree with the FP64 drop-in's physical-space
    sums to the FP32 rounding of the field."""
    cfg = dict(nx=32, ny=24, nz=40, i_strat=1, buoy_fac_z=1.0, lapse=1.0, vis=1e-3, i_cfl=1, cfl0=0.5)
    o = O.Oracle(**cfg)
    u = o.init_random(13)
    stats = []
    for prec in (64, 32):
        g = SamGpu(precision=prec, **cfg)
        g.upload(u)
        g.stage(1)
        stats.append(g.stats())
        g.close()
    s64, s32 = stats
    # the mean is zero up to round-off: compare it on the rms velocity's scale
    rms = np.sqrt(np.abs(s64["u_var"]).max())
    assert np.abs(s32["u_avg"] - s64["u_avg"]).max() <= 1e-6 * rms
    for key in ("u_var", "u_max"):
        scale = np.abs(s64[key]).max()
        assert np.abs(s32[key] - s64[key]).max() <= 1e-6 * scale, key
    assert abs(s32["energy"] - s64["energy"]) <= 1e-6 * s64["energy"]
    assert abs(s32["dt"] - s64["dt"]) <= 1e-6 * s64["dt"]


@pytest.mark.parametrize("n_dealias", [0, 1, 2])
def test_dealias_variants(gpu_lib, n_dealias):
    """The three truncation rules of init.f:49-62 (none, 2/3 in x, y, z;
    2/3 in y and z only) through full resident steps."""
    cfg = dict(nx=24, ny=20, nz=30, i_strat=1, n_dealias=n_dealias, vis=5e-3, buoy_fac_z=1.0, lapse=1.0,
               i_cfl=1, cfl0=0.3)
    g, o = SamGpu(**cfg), O.Oracle(**cfg)
    u = o.init_random(5)
    g.upload(u)
    r = o.wave(o.d.lr)
    o.steps(u, r, 5)
    g.step(5)
    ug = g.download()
    for n in range(o.d.lu):
        assert relerr(ug[..., n], u[..., n]) < TOL_RUN, (n_dealias, n)


def test_nonfinite_field_is_reported(gpu_lib):
    """A NaN planted in the host field before upload: vel_max flags it, the
    CFL dt is not replaced by a value computed from it, and the call itself
    still succeeds (the host decides, as stop_on_error.f would)."""
    for prec in (64, 32):
        cfg = dict(nx=16, ny=16, nz=16, i_cfl=1, cfl0=0.5, dt0=0.02, precision=prec)
        g = SamGpu(**cfg)
        g.init_taylor_green()
        u = g.download()
        u[3, 2, 1, 0] = complex(np.nan, 0.0)
        g.upload(u)
        g.step(1)
        st = g.stats()
        assert st["nonfinite"] == 1, prec
        assert st["dt"] == 0.02, prec
        g.close()


def test_unsupported_lengths_are_rejected(gpu_lib):
    from sam_gb300 import SamGpuError
    for nx, ny, nz in ((14, 16, 16), (16, 22, 16), (16, 16, 2048)):
        with pytest.raises(SamGpuError, match="EINVAL"):
            SamGpu(nx=nx, ny=ny, nz=nz)


@pytest.mark.parametrize("prec", [64, 32])
def test_autotune_leaves_the_state(gpu_lib, prec):
    """The autotuner times the passes on the resident state and puts u, r, p,
    the scalar state (time, dt, statistics) back as they were."""
    cfg = dict(nx=32, ny=32, nz=32, i_strat=1, i_cfl=1, cfl0=0.5, vis=1e-3, buoy_fac_z=1.0, lapse=1.0,
               precision=prec)
    g = SamGpu(**cfg)
    g.init_random(3, 6, 1.0, 6, 0.1)
    g.step(2)
    u0, r0 = g.download(with_r=True)
    s0 = g.stats()
    g.autotune(1)
    u1, r1 = g.download(with_r=True)
    s1 = g.stats()
    assert np.array_equal(u0, u1)
    assert np.array_equal(r0, r1)
    for key, v in s0.items():
        assert np.array_equal(np.asarray(v), np.asarray(s1[key])), key
    g.close()


def test_set_tiles_rejects_bad_tiles(gpu_lib):
    """sam_gpu_set_tiles: odd x-pass rows and out-of-range tiles are refused
    and leave the tiles as they were; a valid set reads back."""
    g = SamGpu(nx=32, ny=32, nz=32, vis=1e-2, dt0=0.01)
    before = g.tiles()
    for bad in (dict(x_rows=3), dict(z_inv_rows=0), dict(y_fwd_planes=65)):
        with pytest.raises(Exception):
            g.set_tiles(**bad)
        assert g.tiles() == before
    g.set_tiles(z_inv_rows=4, x_rows=2, z_fwd_rows=1)
    t = g.tiles()
    assert (t["z_inv_rows"], t["x_rows"], t["z_fwd_rows"]) == (4, 2, 1)
    g.close()
