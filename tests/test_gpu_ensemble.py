"""Ensembles of independent runs (sam_gpu_ensemble_*): members of different
sizes, precisions and closures advanced by one graph per step give exactly
what each run gives on its own."""
import numpy as np
import pytest

import closure as CL
import oracle as O
from sam_gb300 import SamEnsemble, SamGpu

pytestmark = pytest.mark.gpu

MEMBERS = [
    (dict(nx=32, ny=32, nz=32, i_strat=1, buoy_fac_z=2.0, lapse=1.0, vis=2e-3, i_cfl=1, cfl0=0.5), None),
    (dict(nx=24, ny=16, nz=48, vis=1e-3, dt0=0.005), ("les", 2)),
    (dict(nx=48, ny=48, nz=48, i_strat=1, buoy_fac_z=0.5, lapse=1.0, vis=1e-3, i_cfl=1, cfl0=0.5, precision=32),
     ("les", 3)),
    (dict(nx=16, ny=16, nz=16, vis=1e-2, i_cfl=1, cfl0=0.5), ("force", 3)),
]


def _setup(g, extra, u0, params):
    g.upload(u0)
    if extra and extra[0] == "les":
        if extra[1] == 3:
            g.mlp_set(params)
        g.set_les(extra[1])
    if extra and extra[0] == "force":
        g.set_forcing(extra[1], k_f=2.5, sigma=0.3, t_l=0.5)


def test_ensemble_equals_single_runs(gpu_lib):
    params = CL.init_params(9)
    starts = []
    for cfg, _ in MEMBERS:
        c = dict(cfg)
        c.pop("precision", None)
        starts.append(O.Oracle(**c).init_random(len(starts) + 1, 0, 1.0, 0, 0.1))
    singles = []
    for (cfg, extra), u0 in zip(MEMBERS, starts):
        g = SamGpu(**cfg)
        _setup(g, extra, u0, params)
        g.step(4)
        singles.append((g.download(), g.stats()))
        g.close()
    ens = SamEnsemble([cfg for cfg, _ in MEMBERS])
    try:
        for m, ((cfg, extra), u0) in enumerate(zip(MEMBERS, starts)):
            _setup(ens[m], extra, u0, params)
        ens.step(2)
        ens.step(2)
        for m, (u, st) in enumerate(singles):
            assert np.array_equal(ens[m].download(), u), m
            assert ens[m].stats()["time"] == st["time"]
    finally:
        ens.close()


def test_ensemble_member_selection_errors(gpu_lib):
    ens = SamEnsemble([dict(nx=16, ny=16, nz=16), dict(nx=32, ny=32, nz=32)])
    try:
        assert (ens[0].nx, ens[1].nx) == (16, 32)
        ens[1].init_taylor_green()
        ens[0].init_taylor_green()
        ens.step(1)
        assert ens[0].stats()["time"] > 0 and ens[1].stats()["time"] > 0
    finally:
        ens.close()
    # a single context afterwards works as before
    g = SamGpu(nx=16, ny=16, nz=16)
    g.init_taylor_green()
    g.step(1)
    g.close()


PERSISTENT = [
    (dict(nx=32, ny=32, nz=32, i_strat=1, buoy_fac_z=2.0, lapse=1.0, vis=2e-3, i_cfl=1, cfl0=0.5, precision=32),
     None),
    (dict(nx=64, ny=32, nz=96, i_strat=1, buoy_fac_z=1.0, lapse=1.0, vis=1e-3, i_cfl=1, cfl0=0.5, precision=32),
     None),
    (dict(nx=128, ny=64, nz=64, vis=1e-3, dt0=0.002, precision=32), None),
    (dict(nx=32, ny=32, nz=32, i_strat=1, buoy_fac_z=1.0, lapse=1.0, vis=2e-3, i_cfl=1, cfl0=0.5), None),
    (dict(nx=32, ny=64, nz=32, vis=3e-3, i_cfl=1, cfl0=0.5, precision=32), ("force", 5)),
    (dict(nx=96, ny=96, nz=96, i_strat=1, buoy_fac_z=1.0, lapse=1.0, vis=1e-3, i_cfl=1, cfl0=0.5, nrk_max=2,
          precision=32), None),
]


@pytest.mark.parametrize("persistent", [True, False])
def test_persistent_stage_launch_equals_single_runs(gpu_lib, persistent):
    """The FP32 members without a closure whose lengths are 32, 64, 96 or 128
    (five of the six here: the FP64 member keeps its own branch) advance in
    one persistent launch per RK3 stage; every member ends bit for bit where
    it ends when run alone, with either arrangement."""
    params = CL.init_params(9)
    starts = []
    for cfg, _ in PERSISTENT:
        c = dict(cfg)
        c.pop("precision", None)
        starts.append(O.Oracle(**c).init_random(len(starts) + 11, 6, 1.0, 6, 0.1))
    singles = []
    for (cfg, extra), u0 in zip(PERSISTENT, starts):
        g = SamGpu(**cfg)
        _setup(g, extra, u0, params)
        g.step(3)
        singles.append((g.download(), g.stats()))
        g.close()
    ens = SamEnsemble([cfg for cfg, _ in PERSISTENT])
    try:
        ens.set_persistent(persistent)
        for m, ((cfg, extra), u0) in enumerate(zip(PERSISTENT, starts)):
            _setup(ens[m], extra, u0, params)
        ens.step(1)
        assert ens.persistent_members() == (5 if persistent else 0)
        ens.step(2)
        for m, (u, st) in enumerate(singles):
            assert np.array_equal(ens[m].download(), u), m
            got = ens[m].stats()
            assert got["time"] == st["time"] and got["dt"] == st["dt"], m
            assert np.array_equal(got["u_max"], st["u_max"]), m
    finally:
        ens.close()


def test_ensemble_autotune_per_class(gpu_lib):
    """SamEnsemble.autotune tunes one member per class of branch members and
    copies its tiles and FFT schedules to the rest of the class; members of
    the persistent launch keep their tiles; each member then steps exactly
    as its own run with the same tiles."""
    params = CL.init_params(4)
    les_cfg = dict(nx=32, ny=32, nz=32, i_strat=1, buoy_fac_z=1.0, lapse=1.0, vis=2e-3, i_cfl=1, cfl0=0.5,
                   precision=32)
    small = dict(nx=32, ny=32, nz=32, vis=1e-2, i_cfl=1, cfl0=0.5, precision=32)
    cfgs = [les_cfg, les_cfg, small]
    starts = []
    for c in cfgs:
        c0 = dict(c)
        c0.pop("precision")
        starts.append(O.Oracle(**c0).init_random(len(starts) + 21, 0, 1.0, 0, 0.1))
    ens = SamEnsemble(cfgs)
    try:
        defaults = ens[2].tiles()
        for m in range(3):
            ens[m].upload(starts[m])
        for m in (0, 1):
            ens[m].mlp_set(params)
            ens[m].set_les(3)
        tuned = ens.autotune(2)
        assert list(tuned) == [(32, 32, 32, 32, 3)]
        t0 = dict(tuned[(32, 32, 32, 32, 3)])
        sched = t0.pop("fft_schedule")
        assert ens[1].tiles() == t0 and ens[1].fft_schedule() == sched
        assert ens[2].tiles() == defaults
        ens.step(2)
        assert ens.persistent_members() == 1
        out = [(ens[m].download(), ens[m].stats()["dt"]) for m in range(3)]
    finally:
        ens.close()
    for m in range(3):
        g = SamGpu(**cfgs[m])
        g.upload(starts[m])
        if m < 2:
            g.mlp_set(params)
            g.set_les(3)
            g.set_tiles(**t0)
            g.set_fft_schedule(sched)
        g.step(2)
        assert np.array_equal(g.download(), out[m][0]), m
        assert g.stats()["dt"] == out[m][1]
        g.close()
