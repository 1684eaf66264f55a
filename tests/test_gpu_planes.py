"""Planes output path (sam.f:145-166, write_planes.f) of the GPU context
against the oracle, and the n_var = 2 Nu variants of the backward transform
chain that this output step calls (sam.f:159, 228-232)."""
import numpy as np
import pytest

import oracle as O
from sam_gb300 import SamGpu, SamGpuError

pytestmark = pytest.mark.gpu

PLANES = dict(k_xy=[1, 5, 32], j_xz=[3, 16], i_yz=[1, 24])


def _stepped(cfg, precision=64, seed=5):
    """A GPU context one step into a run (so p = r(Lu+1) exists) and the
    oracle on the same configuration."""
    g, o = SamGpu(precision=precision, **cfg), O.Oracle(**cfg)
    g.upload(o.init_random(seed))
    g.step(1)
    u, r = g.download(with_r=True)
    return g, o, u, r


def _compare(got, ref, lu, rel):
    for key in ("xy", "xz", "yz"):
        assert got[key].shape == ref[key].shape, key
        if got[key].size == 0:
            continue
        for s in range(2 * lu):
            scale = max(np.abs(ref[key][:, :, s, :]).max(), 1e-300)
            err = np.abs(got[key][:, :, s, :] - ref[key][:, :, s, :]).max()
            assert err <= rel * scale, (key, s, err / scale)
    scale = np.abs(ref["mean"]).max()
    assert np.abs(got["mean"] - ref["mean"]).max() <= rel * max(scale, 1e-300)


@pytest.mark.parametrize("strat", [0, 1])
def test_planes_match_oracle(gpu_lib, strat):
    cfg = dict(nx=24, ny=16, nz=32, i_strat=strat, buoy_fac_z=1.0 * strat, lapse=1.0 * strat, vis=1e-3)
    g, o, u, r = _stepped(cfg)
    lu = o.d.lu
    ref = o.planes(u, r[..., lu:lu + 1], **PLANES)
    got = g.planes(**PLANES)
    _compare(got, ref, lu, 1e-12)


def test_planes_fp32_bulk(gpu_lib):
    cfg = dict(nx=32, ny=32, nz=32, i_strat=1, buoy_fac_z=1.0, lapse=1.0, vis=1e-3)
    g, o, u, r = _stepped(cfg, precision=32)
    lu = o.d.lu
    ref = o.planes(u, r[..., lu:lu + 1], **PLANES)
    _compare(g.planes(**PLANES), ref, lu, 2e-5)


def test_planes_leave_state_and_subsets(gpu_lib):
    """Only some orientations, and the resident state is unchanged."""
    cfg = dict(nx=24, ny=16, nz=32, i_strat=1, buoy_fac_z=1.0, lapse=1.0, vis=1e-3)
    g, o, u, r = _stepped(cfg)
    lu = o.d.lu
    got = g.planes(i_yz=[7])
    ref = o.planes(u, r[..., lu:lu + 1], i_yz=[7])
    assert got["xy"].shape[-1] == 0 and got["xz"].shape[-1] == 0
    _compare(got, ref, lu, 1e-12)
    u2, r2 = g.download(with_r=True)
    assert np.array_equal(u2, u) and np.array_equal(r2, r)


def test_planes_reject_bad_indices(gpu_lib):
    g = SamGpu(nx=16, ny=16, nz=16)
    with pytest.raises(SamGpuError, match="EINVAL"):
        g.planes(k_xy=[0])
    with pytest.raises(SamGpuError, match="EINVAL"):
        g.planes(j_xz=[17])
    with pytest.raises(SamGpuError, match="EINVAL"):
        g.planes(i_yz=list(range(1, 18)))


def test_backward_chain_two_nu_fields(gpu_lib):
    """z_trans_b, x2z_decomp and xy_trans_b with n_var = 2 Nu, as the output
    step calls them (sam.f:159, 228-232)."""
    cfg = dict(nx=24, ny=16, nz=32, i_strat=1)
    g, o = SamGpu(**cfg), O.Oracle(**cfg)
    lu = o.d.lu
    u = o.wave(2 * lu)
    u[..., :lu] = o.init_random(1)
    u[..., lu:] = o.init_random(2)
    zo, zg = o.z_trans_b(u, 2 * lu), g.z_trans_b(u, 2 * lu)
    assert np.abs(zg - zo).max() <= 1e-13 * np.abs(zo).max()
    xo, xg = o.x2z_decomp(zo, 2 * lu), g.x2z_decomp(zo, 2 * lu)
    m = o.d.nx_min
    assert np.abs(xg[:, :m] - xo[:, :m]).max() <= 1e-15 * np.abs(xo).max()
    po, pg = o.xy_trans_b(xo.copy(order="F"), 2 * lu), g.xy_trans_b(xo, 2 * lu)
    assert np.abs(pg - po).max() <= 1e-13 * np.abs(po).max()
