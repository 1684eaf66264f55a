"""The numpy restatement of the closure network (oracle/closure.py) checked
on the CPU: BF16 rounding, and its analytic gradient against central finite
differences of the unrounded network."""
import numpy as np

import closure as CL


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.001953125, 1.005859375, -3.14159265, 0.0, 65504.0], dtype=np.float32)
    r = CL.bf16(x)
    # BF16 spacing at 1 is 2^-7: 1 + 2^-8 is a tie (even mantissa wins: 1),
    # 1 + 2^-9 rounds down, 1 + 3 * 2^-9 rounds up to 1 + 2^-7
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 and r[3] == 1.0078125
    assert abs(r[4] + 3.140625) < 1e-7 and r[5] == 0.0 and r[6] == 65536.0
    # BF16 keeps 8 significant bits: relative error at most 2^-9
    v = np.random.default_rng(0).standard_normal(1000).astype(np.float32)
    assert np.all(np.abs(CL.bf16(v) - v) <= np.abs(v) * 2.0 ** -8)


def test_gradient_against_finite_differences():
    rng = np.random.default_rng(3)
    p = CL.init_params(1).astype(np.float64)
    p[CL.OFF_W3:CL.OFF_B3] *= 20  # make the output layer matter
    x = rng.standard_normal((64, CL.N_IN))
    y = np.abs(rng.standard_normal((64, 2))) * 0.02
    g, _ = CL.grad(p, x, y, rnd=False)
    idx = np.concatenate([rng.choice(CL.N_PARAMS, 40, replace=False), [CL.OFF_B3, CL.OFF_B3 + 1, CL.OFF_B1]])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp = CL.grad(pp, x, y, rnd=False)[1]
        lm = CL.grad(pm, x, y, rnd=False)[1]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(abs(fd), 1e-8) + 1e-12, (i, fd, g[i])


def test_invariants_of_simple_flows():
    """Pure strain, pure rotation and stratification give the invariants
    their definitions predict."""
    import oracle as O
    # axisymmetric strain diag(2, -1, -1): |S|^2 = 2 * 6 = 12, tr(S^3) = 6
    S = np.array([2.0, 0, -1.0, 0, 0, -1.0])
    f = O.closure_invariants(S, np.zeros(3), np.zeros(3), dsq=1.0, nu=1.0)
    assert abs(f[0]) < 1e-7 and abs(f[1] - 6 / 12 ** 1.5) < 1e-6 and abs(f[6] + 1 / 12 ** 0.5) < 1e-6
    assert abs(f[10] - np.log1p(12 ** 0.5)) < 1e-6 and f[11] == 0
    # strain plus rotation about z: w = (0, 0, 2), |w|^2/|S|^2 = 4/12
    f = O.closure_invariants(S, np.zeros(3), np.array([0, 0, 2.0]), dsq=1.0, nu=1.0)
    assert abs(f[0] - np.log1p(4 / 12)) < 1e-6
    assert abs(f[2] - (-1 * 4) / (12 ** 0.5 * 4)) < 1e-6 and abs(f[7] - 2 / (12 ** 0.5 + 2)) < 1e-6
    # stable stratification dT/dz = 0.5 with b = 2, N^2 = 3
    f = O.closure_invariants(S, np.array([0, 0, 0.5]), np.zeros(3), bz=2.0, n2=3.0, dsq=1.0, nu=1.0)
    assert abs(f[3] - np.log1p(3 / 12)) < 1e-6 and abs(f[4] - np.arcsinh(1 / 12)) < 1e-6 and f[5] == 0
    assert abs(f[8] - (-1 * 0.25) / (12 ** 0.5 * 0.25)) < 1e-6


def test_zero_network_is_smagorinsky():
    """With every parameter zero the network returns C = 0.02 ln 2 for both
    coefficients, so the learned closure (model 3) must reproduce the
    Smagorinsky closure (model 1) with that constant and Pr_t = 1 exactly."""
    import oracle as O
    c0 = float(np.float32(0.02) * np.float32(np.log1p(np.float32(1.0))))
    cfg = dict(nx=16, ny=16, nz=24, i_strat=1, buoy_fac_z=1.0, lapse=1.0, vis=1e-4, dt0=0.01)
    us = []
    for model in (1, 3):
        o = O.Oracle(**cfg)
        u = o.init_random(4, 0, 1.0, 0, 0.1)
        o.mlp_set(np.zeros(CL.N_PARAMS, np.float32))
        o.set_les(model, c_smag=c0, pr_t=1.0)
        r = o.wave(o.d.lr)
        o.steps(u, r, 2)
        us.append(u)
    assert np.array_equal(us[0], us[1])


def test_training_targets_recover_a_known_eddy_viscosity_and_diffusivity():
    """closure_data.targets: filtered fields whose subgrid stress is exactly
    -2 nu0 S (S traceless) and whose subgrid flux is exactly -kappa0 grad T
    give C_nu* = nu0 / (delta^2 |S|) and C_kappa* = kappa0 / (delta^2 |S|)
    (clipped to [0, C_MAX] in the first output, unclipped in the second)."""
    from sam_gb300 import closure_data as CD

    rng = np.random.default_rng(4)
    shp = (6, 5, 4)
    lu, dsq, nu0, kap0 = 4, 0.02, 3e-4, 5e-4
    ub = rng.standard_normal(shp + (3,))
    tb = rng.standard_normal(shp)
    S = rng.standard_normal(shp + (6,))  # product order S11 S12 S22 S13 S23 S33
    S[..., 5] = -(S[..., 0] + S[..., 2])
    gT = rng.standard_normal(shp + (3,))
    pairs = [(0, 0), (0, 1), (1, 1), (0, 2), (1, 2), (2, 2)]
    filt = np.zeros(shp + (lu + 9,))
    filt[..., :3] = ub
    filt[..., 3] = tb
    for m, (a, b) in enumerate(pairs):
        filt[..., lu + m] = ub[..., a] * ub[..., b] - 2 * nu0 * S[..., m]
    for a in range(3):
        filt[..., lu + 6 + a] = ub[..., a] * tb - kap0 * gT[..., a]
    grads = np.concatenate([S, gT], axis=-1)
    clipped, raw, smag = CD.targets(np.asfortranarray(filt), np.asfortranarray(grads), lu, dsq)
    ss = sum(w * S[..., m] ** 2 for m, w in enumerate([1, 2, 1, 2, 2, 1]))
    smag_ref = np.sqrt(2 * ss).ravel(order="F")
    np.testing.assert_allclose(smag, smag_ref, rtol=1e-12)
    np.testing.assert_allclose(raw[:, 0], nu0 / (dsq * smag_ref), rtol=1e-9)
    np.testing.assert_allclose(raw[:, 1], kap0 / (dsq * smag_ref), rtol=1e-9)
    assert clipped.dtype == np.float32 and clipped.min() >= 0 and clipped.max() <= CD.C_MAX
    np.testing.assert_allclose(clipped, np.clip(raw, 0, CD.C_MAX), rtol=1e-6)
