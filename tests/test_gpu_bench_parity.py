"""Parity with the oracle at the benchmark configurations (sam.f:122-326).

* the 256^3 gravity-wave packet the headline number is measured on (N = 2,
  nu = kappa = 1e-4, CFL 0.5): two full RK3 steps from the same start, FP64
  and the double-float form within 1e-12 per field, the FP32 bulk form's
  error bounded;
* the 128^3 stratified decaying turbulence (N = 1, Pr = 1, nu = 1/800,
  k^4 exp(-2 (k/4)^2) start at rms 1, CFL 0.5) with seeds 0, 1 and 2 over
  60 CFL steps: FP64 and double-float within 1e-12 per field, dt and time
  to 1e-12.

Errors are relative to each field's largest coefficient (Nz_min rows).
"""
import numpy as np
import pytest

import oracle as O
from sam_gb300 import SamGpu

pytestmark = pytest.mark.gpu

TOL_RUN = 1e-12


def field_errors(ug, uo, nz_min):
    return [float(np.abs(ug[:nz_min, ..., n] - uo[:nz_min, ..., n]).max() / np.abs(uo[:nz_min, ..., n]).max())
            for n in range(uo.shape[-1])]


def packet_cfg(n=256):
    return dict(nx=n, ny=n, nz=n, i_strat=1, i_cfl=1, cfl0=0.5, vis=1e-4, pr=1.0, dt0=1e-3, buoy_fac_z=4.0,
                lapse=1.0)


def test_headline_packet_256_two_steps(gpu_lib):
    cfg = packet_cfg()
    g = SamGpu(**cfg)
    g.init_packet(1, (8, 0, 16), np.pi / 4, 0.05, 0.01)
    u0 = g.download()
    o = O.Oracle(**cfg)
    uo = o.init_packet(1, (8, 0, 16), np.pi / 4, 0.05, 0.01)
    assert np.abs(uo - u0).max() / np.abs(u0).max() < 1e-13  # the same seeded start
    u = u0.copy(order="F")
    r = o.wave(o.d.lr)
    o.steps(u, r, 2)
    g.step(2)
    ug = g.download()
    err = field_errors(ug, u, o.d.nz_min)
    print("256^3 packet, 2 steps, FP64 error per field:", err)
    assert max(err) < TOL_RUN, err
    so, sg = o.stats(), g.stats()
    assert abs(sg["dt"] - so["dt"]) <= 1e-13 * so["dt"]
    assert abs(sg["time"] - so["time"]) <= 1e-12
    assert g.div_check()["div_max"] < 1e-11
    g.close()
    # the double-float form from the same start, at the FP64 bar
    gdd = SamGpu(precision=48, **cfg)
    gdd.upload(u0)
    gdd.step(2)
    edd = field_errors(gdd.download(), u, o.d.nz_min)
    print("256^3 packet, 2 steps, double-float error per field:", edd)
    assert max(edd) < TOL_RUN, edd
    assert abs(gdd.stats()["dt"] - so["dt"]) <= 1e-13 * so["dt"]
    gdd.close()
    # the FP32 bulk form from the same start
    g32 = SamGpu(precision=32, **cfg)
    g32.upload(u0)
    g32.step(2)
    e32 = field_errors(g32.download(), u, o.d.nz_min)
    print("256^3 packet, 2 steps, FP32 bulk error per field:", e32)
    assert max(e32) < 1e-5, e32
    g32.close()
    o.close()


@pytest.mark.parametrize("precision", [64, 48])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_stratified_128_config_60_cfl_steps(gpu_lib, seed, precision):
    cfg = dict(nx=128, ny=128, nz=128, i_strat=1, i_cfl=1, cfl0=0.5, vis=1.0 / 800, pr=1.0, buoy_fac_z=1.0,
               lapse=1.0)
    o = O.Oracle(**cfg)
    u = o.init_random(seed, 6, 1.0, 6, 0.1)
    g = SamGpu(precision=precision, **cfg)
    g.init_random(seed, 6, 1.0, 6, 0.1)
    # the device's seeded start agrees with the oracle's to the rounding of
    # its sines and cosines; the run itself starts from the oracle's field
    assert np.abs(g.download() - u).max() / np.abs(u).max() < 1e-13
    g.upload(u)
    r = o.wave(o.d.lr)
    o.steps(u, r, 60)
    g.step(60)
    err = field_errors(g.download(), u, o.d.nz_min)
    print(f"128^3 stratified seed {seed}, 60 CFL steps, precision {precision}, error per field:", err)
    assert max(err) < TOL_RUN, err
    so, sg = o.stats(), g.stats()
    assert abs(sg["dt"] - so["dt"]) <= 1e-12 * so["dt"]
    assert abs(sg["time"] - so["time"]) <= 1e-12 * max(1.0, so["time"])
    g.close()
    o.close()
