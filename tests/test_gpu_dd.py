"""The double-float form (precision 48: every transform, product and update
in FP32 pairs on the FP32 pipe, vel_max's sums and the integrating factor's
exponentials in FP64) against the FP64 oracle: full runs at the FP64 drop-in's
bar, within 1e-12 per field (Taylor-Green 64^3 x 200 steps, stratified CFL
turbulence, the three dealias rules, the input.dat wave); single stages
within 2e-13 of the field maximum on every grid and FFT path (the pairs carry
about 48 bits, so a stage of the 512- and 1024-point transforms lands near
1.2e-13, against the FP64 drop-in's 1e-13 per routine).
"""
import os

import numpy as np
import pytest

import oracle as O
from sam_gb300 import SamGpu, SamGpuError
from test_gpu_parity import GOLD, GRIDS, relerr

pytestmark = pytest.mark.gpu

DD = 48
TOL_ROUTINE = 2e-13
TOL_RUN = 1e-12


def pair(**kw):
    base = dict(vis=1e-2, pr=0.7, dt0=0.01, buoy_fac_z=1.0 if kw.get("i_strat") else 0.0,
                lapse=1.0 if kw.get("i_strat") else 0.0)
    base.update(kw)
    return SamGpu(precision=DD, **base), O.Oracle(**base)


@pytest.mark.parametrize("grid", GRIDS)
def test_dd_resident_stages(gpu_lib, grid):
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
    g.close()


@pytest.mark.parametrize("grid", [g for g in GRIDS if 256 in (g["nx"], g["ny"], g["nz"])])
def test_dd_resident_stages_stockham_schedule(gpu_lib, grid):
    g, o = pair(**grid)
    d = o.d
    g.set_fft_schedule([1, 1, 1, 1, 1])
    u = o.init_random(43)
    g.upload(u)
    r = o.wave(d.lr)
    for nrk in (1, 2, 3):
        o.stage(u, r, nrk)
        g.stage(nrk)
        ug = g.download()
        for n in range(d.lu):
            assert relerr(ug[: d.nz_min, ..., n], u[: d.nz_min, ..., n]) < TOL_ROUTINE, (nrk, n)
    g.close()


def test_dd_taylor_green_64_200_steps(gpu_lib):
    cfg = dict(nx=64, ny=64, nz=64, vis=1.0 / 400, dt0=0.01)
    g, o = SamGpu(precision=DD, **cfg), O.Oracle(**cfg)
    u = o.init_taylor_green()
    g.init_taylor_green()
    r = o.wave(o.d.lr)
    o.steps(u, r, 200)
    g.step(200)
    ug = g.download()
    for n in range(3):
        err = relerr(ug[: o.d.nz_min, ..., n], u[: o.d.nz_min, ..., n]) if n < 2 else \
            np.abs(ug[..., n] - u[..., n]).max() / np.abs(u[..., :2]).max()
        print("Taylor-Green 64^3, 200 steps, double-float error of field", n, err)
        assert err < TOL_RUN, (n, err)
    assert abs(g.stats()["time"] - 2.0) < 1e-12
    g.close()


def test_dd_stratified_cfl_run(gpu_lib):
    cfg = dict(nx=32, ny=32, nz=32, i_strat=1, i_cfl=1, cfl0=0.5, vis=1.0 / 800, pr=1.0, buoy_fac_z=1.0,
               lapse=1.0)
    g, o = SamGpu(precision=DD, **cfg), O.Oracle(**cfg)
    u = o.init_random(0, 6, 1.0, 6, 0.1)
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
    # vel_max's statistics (u_max from the pairs, the sums from wave space)
    np.testing.assert_allclose(sg["u_max"][:4], so["u_max"][:4], rtol=1e-13)
    np.testing.assert_allclose(sg["u_var"][:4], so["u_var"][:4], rtol=1e-12)
    assert abs(sg["energy"] - so["energy"]) <= 1e-12 * so["energy"]
    g.close()


def test_dd_gravity_wave_input_dat(gpu_lib):
    gd = GOLD["gw_input_dat"]
    cfg = dict(nx=gd["nx"], ny=gd["ny"], nz=gd["nz"], xl=gd["xl"], yl=gd["yl"], zl=gd["zl"], i_strat=1,
               vis=gd["vis"], dt0=gd["dt"], buoy_fac_z=gd["grav"] / gd["to"], lapse=gd["lapse0"])
    g, o = SamGpu(precision=DD, **cfg), O.Oracle(**cfg)
    u0 = o.init_gw_plane(gd["amplitude"], gd["lambda_x"], gd["lambda_z"], gd["omega_i"], gd["k_w"], gd["m_w"],
                         gd["lapse0"], gd["uo"])
    g.upload(u0)
    g.step(gd["n_steps"])
    ug = g.download()
    amp = complex(gd["rk3_amplification_re"], gd["rk3_amplification_im"])
    assert np.abs(ug - u0 * amp).max() / np.abs(u0).max() < 1e-12
    g.close()


@pytest.mark.parametrize("n_dealias", [0, 1, 2])
def test_dd_dealias_variants(gpu_lib, n_dealias):
    cfg = dict(nx=24, ny=20, nz=30, i_strat=1, n_dealias=n_dealias, vis=5e-3, buoy_fac_z=1.0, lapse=1.0,
               i_cfl=1, cfl0=0.3)
    g, o = SamGpu(precision=DD, **cfg), O.Oracle(**cfg)
    u = o.init_random(5)
    g.upload(u)
    r = o.wave(o.d.lr)
    o.steps(u, r, 5)
    g.step(5)
    ug = g.download()
    for n in range(o.d.lu):
        assert relerr(ug[..., n], u[..., n]) < TOL_RUN, (n_dealias, n)
    g.close()


def test_dd_diagnostics_and_restart(gpu_lib, tmp_path):
    """spectra, div_check and cl_energy read FP64 copies of the pairs; a
    restart file written from the pairs reads back to the same state."""
    cfg = dict(nx=32, ny=24, nz=40, i_strat=1, i_les=1, vis=1e-3, buoy_fac_z=1.0, lapse=1.0)
    g, o = SamGpu(precision=DD, **cfg), O.Oracle(**cfg)
    u = o.init_random(5)
    g.upload(u)
    r = o.wave(o.d.lr)
    o.stage(u, r, 1)
    g.stage(1)
    so, sg = o.spectra(u, r), g.spectra()
    for key in ("ek", "tk", "dk", "vt", "sample"):
        np.testing.assert_allclose(sg[key], so[key], rtol=1e-11, atol=1e-14 * np.abs(so[key]).max())
    assert g.div_check()["div_max"] < 1e-12
    assert abs(g.cl_energy() - o.cl_energy(u)) <= 1e-11 * o.cl_energy(u)
    f = str(tmp_path / "vel.000001")
    before = g.download()
    g.write_field(f)
    g.upload(np.zeros_like(before))
    g.read_field(f)
    assert np.array_equal(g.download(), before)
    g.close()


def test_dd_nonfinite_field_is_reported(gpu_lib):
    g = SamGpu(nx=16, ny=16, nz=16, i_cfl=1, cfl0=0.5, dt0=0.02, precision=DD)
    g.init_taylor_green()
    u = g.download()
    u[3, 2, 1, 0] = complex(np.nan, 0.0)
    g.upload(u)
    g.step(1)
    st = g.stats()
    assert st["nonfinite"] == 1
    assert st["dt"] == 0.02
    g.close()


def test_dd_autotune_leaves_the_state(gpu_lib):
    cfg = dict(nx=32, ny=32, nz=32, i_strat=1, i_cfl=1, cfl0=0.5, vis=1e-3, buoy_fac_z=1.0, lapse=1.0,
               precision=DD)
    g = SamGpu(**cfg)
    g.init_random(3, 6, 1.0, 6, 0.1)
    g.step(2)
    u0, r0 = g.download(with_r=True)
    s0 = g.stats()
    g.autotune(1)
    u1, r1 = g.download(with_r=True)
    assert np.array_equal(u0, u1) and np.array_equal(r0, r1)
    for key, v in s0.items():
        assert np.array_equal(np.asarray(v), np.asarray(g.stats()[key])), key
    g.close()


def test_dd_plain_step_only(gpu_lib):
    """The closures, the OU forcing and the planes output are not part of the
    double-float form: asking for them is an error, not a silent FP64 run."""
    g = SamGpu(nx=16, ny=16, nz=16, i_strat=1, buoy_fac_z=1.0, lapse=1.0, precision=DD)
    for call in (lambda: g.set_les(1), lambda: g.set_forcing(1, 2.5, 0.1, 1.0)):
        with pytest.raises(SamGpuError, match="EUNSUPPORTED"):
            call()
    g.close()
