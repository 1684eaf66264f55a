"""Spectral forcing (force.f) and the restart files (write_field.f,
read_field.f, write_header.f, read_header.f) of the GPU context against the
oracle, including the failure paths the reference checks on the host."""
import os

import numpy as np
import pytest

import oracle as O
from sam_gb300 import SamGpu, SamGpuError

pytestmark = pytest.mark.gpu


def test_force_matches_oracle(gpu_lib):
    cfg = dict(nx=32, ny=24, nz=40, vis=1e-3)
    g, o = SamGpu(**cfg), O.Oracle(**cfg)
    u = o.init_random(12, 6, 1.0, 6, 0.0)
    r = o.wave(o.d.lr)
    ek_0 = o.spectra(u, r)["ek"].copy()
    o.steps(u, r, 3)  # let the shells drift
    g.upload(u)
    o.force(u, ek_0, 2)
    g.force(ek_0, 2)
    ug = g.download()
    assert np.abs(ug - u).max() <= 1e-14 * np.abs(u).max()
    ek = o.spectra(u, r)["ek"]
    np.testing.assert_allclose(ek[1:3], ek_0[1:3], rtol=1e-13)


def test_restart_round_trip_between_gpu_and_oracle(gpu_lib, tmp_path):
    cfg = dict(nx=24, ny=16, nz=32, i_strat=1, buoy_fac_z=1.0, lapse=1.0, dt0=0.02)
    g, o = SamGpu(**cfg), O.Oracle(**cfg)
    u = o.init_random(3)
    g.upload(u)
    g.step(2)
    f1 = str(tmp_path / "vel.000002")
    h1 = str(tmp_path / "header.000002")
    g.write_field(f1)
    g.write_header(h1, 2)
    # the oracle reads the GPU's file: the same modes, padding rows zero
    uo = o.read_field(f1)
    assert np.array_equal(uo, g.download())
    # a fresh context restarts from it and continues identically
    st = g.stats()
    g2 = SamGpu(**cfg)
    g2.read_field(f1)
    assert g2.read_header(h1) == 2
    s2 = g2.stats()
    assert s2["time"] == st["time"] and s2["dt"] == st["dt"]
    assert np.array_equal(g2.download(), uo)
    # and the oracle's own file is read back by the GPU bit for bit
    f2 = str(tmp_path / "vel.oracle")
    o.write_field(f2, u)
    g2.read_field(f2)
    assert np.array_equal(g2.download(), u)


def test_restart_failure_paths(gpu_lib, tmp_path):
    cfg = dict(nx=16, ny=16, nz=16)
    g = SamGpu(**cfg)
    g.init_taylor_green()
    f = str(tmp_path / "vel.000000")
    g.write_field(f)
    # truncated file: read_field.f:26-32 rejects the size
    with open(f, "r+b") as fh:
        fh.truncate(os.path.getsize(f) - 16)
    with pytest.raises(SamGpuError, match="not of correct size"):
        g.read_field(f)
    o = O.Oracle(**cfg)
    assert o.read_field(f) == -2
    # a header whose grid differs: read_header.f:25-38 stops on fixed parameters
    h = str(tmp_path / "header.000000")
    g.write_header(h, 0)
    text = open(h).read().replace(" Nx 16", " Nx 32")
    open(h, "w").write(text)
    with pytest.raises(SamGpuError, match="nx differs"):
        g.read_header(h)


@pytest.mark.parametrize("strat", [0, 1])
def test_ou_forcing_matches_oracle(gpu_lib, strat):
    """Stochastic low-wavenumber forcing inside sam_gpu_step against the
    oracle's so_steps with the same seed, over several steps with CFL dt."""
    cfg = dict(nx=24, ny=16, nz=32, i_strat=strat, buoy_fac_z=1.0 * strat, lapse=1.0 * strat, vis=1e-3,
               i_cfl=1, cfl0=0.5)
    g, o = SamGpu(**cfg), O.Oracle(**cfg)
    u = o.init_random(4)
    r = o.wave(o.d.lr)
    g.upload(u)
    assert g.set_forcing(11, k_f=2.5, sigma=0.5, t_l=0.3) == o.set_forcing(11, k_f=2.5, sigma=0.5, t_l=0.3)
    o.steps(u, r, 6)
    g.step(6)
    ug = g.download()
    for n in range(o.d.lu):
        assert np.abs(ug[..., n] - u[..., n]).max() <= 1e-12 * np.abs(u[..., n]).max(), n


def test_ou_forcing_off_and_restart(gpu_lib):
    cfg = dict(nx=16, ny=16, nz=16, vis=1e-3)
    g = SamGpu(**cfg)
    g.init_taylor_green()
    u0 = g.download()
    g.set_forcing(1, k_f=2.5, sigma=0.5, t_l=1.0)
    g.set_forcing(1, k_f=0.0)
    g.step(2)
    g2 = SamGpu(**cfg)
    g2.init_taylor_green()
    g2.step(2)
    assert np.array_equal(g.download(), g2.download())
    # a new set_forcing restarts the amplitude sequence from step 0
    g.upload(u0)
    g.set_forcing(5, k_f=2.0, sigma=0.2, t_l=1.0)
    g.step(2)
    a = g.download()
    g.upload(u0)
    g.set_forcing(5, k_f=2.0, sigma=0.2, t_l=1.0)
    g.step(2)
    assert np.array_equal(g.download(), a)
    with pytest.raises(SamGpuError, match="EINVAL"):
        g.set_forcing(5, k_f=2.0, sigma=0.2, t_l=0.0)
