"""The oracle pinned against the reference's own known-answer tests (CPU)."""
import json
import os

import numpy as np
import pytest

import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "kats.json")))


def small(tol, x):
    # fft.f:2899 SMALL(EX) = TRUNC(1.0 + TOL*ABS(EX)) - 1.0 in single precision
    return np.float32(1.0 + tol * abs(x)) - np.float32(1.0) == 0.0


def test_tfftpk_rfftf_rfftb():
    """FFTPACK's TFFTPK (fft.f:2838-3011) at N=36, tolerance as there."""
    n, tol = GOLD["tfftpk"]["n"], GOLD["tfftpk"]["tol"]
    r = O.fft_line(np.ones(n), "rfftf")
    err = max(abs(n - r[0]), np.abs(r[1:]).max())
    assert small(tol, err)
    d = np.zeros(n)
    d[0] = 1.0
    b = O.fft_line(d, "rfftb")
    assert small(tol, np.abs(1.0 - b).max())
    # and much tighter than TFFTPK's single-precision bar
    assert err < 1e-13 and np.abs(1.0 - b).max() < 1e-14


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 12, 16, 24, 36, 64, 72, 96, 100, 128, 256, 384, 512])
def test_fft_conventions_against_numpy(n):
    """cfftf = sum c e^{-i}, cfftb = sum c e^{+i}, unnormalised (fft.f:24-60);
    rfftf packing r(1)=DC, r(2k-2)=Re, r(2k-1)=Im, r(n)=Nyquist (fft.f:2350-2403)."""
    rng = np.random.default_rng(n)
    c = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    f = O.fft_line(c, "cfftf")
    np.testing.assert_allclose(f, np.fft.fft(c), rtol=0, atol=1e-13 * n)
    b = O.fft_line(c, "cfftb")
    np.testing.assert_allclose(b, np.fft.ifft(c) * n, rtol=0, atol=1e-13 * n)
    x = rng.standard_normal(n)
    rf = O.fft_line(x, "rfftf")
    X = np.fft.rfft(x)
    packed = np.zeros(n)
    packed[0] = X[0].real
    for k in range(1, (n + 1) // 2):
        packed[2 * k - 1] = X[k].real
        packed[2 * k] = X[k].imag
    if n % 2 == 0 and n > 1:
        packed[n - 1] = X[n // 2].real
    np.testing.assert_allclose(rf, packed, rtol=0, atol=1e-13 * n)
    rb = O.fft_line(rf, "rfftb")
    np.testing.assert_allclose(rb, n * x, rtol=0, atol=1e-12 * n)


@pytest.mark.parametrize("dims,strat", [((16, 16, 16), 0), ((12, 8, 24), 1), ((72, 1, 24), 1), ((32, 48, 20), 1)])
def test_tst_transpose_round_trip(dims, strat):
    """tst_transpose.f:98-146: z_trans_b -> x2z -> xy_trans_b -> xy_trans_f ->
    z2x -> z_trans_f reproduces every mode to 1e-15."""
    nx, ny, nz = dims
    o = O.Oracle(nx=nx, ny=ny, nz=nz, i_strat=strat)
    d = o.d
    u = o.init_random(11)
    zb = o.z_trans_b(u, d.lu)
    xy = o.x2z_decomp(zb, d.lu)
    ph = o.xy_trans_b(xy, d.lu)
    w = o.xy_trans_f(ph, d.lu)
    o.z_trans_f(w, d.lu)
    diff = np.abs(w[: d.nz_min] - u[: d.nz_min])
    assert (diff > GOLD["tst_transpose"]["tol"]).sum() == 0, diff.max()


def test_physical_synthesis_matches_numpy():
    """The backward chain equals numpy's inverse real FFT of the same modes."""
    nx, ny, nz = 16, 12, 20
    o = O.Oracle(nx=nx, ny=ny, nz=nz, i_strat=1)
    d = o.d
    u = o.init_random(3)
    ph = o.xy_trans_b(o.x2z_decomp(o.z_trans_b(u, d.lu), d.lu), d.lu)
    for n in range(d.lu):
        spec = np.zeros((nz, ny, nx // 2 + 1), complex)
        for i in range(d.nx_min):
            for j in range(d.ny_min):
                ky = j if j <= d.ky_max else j - d.ny_min
                for k in range(d.nz_min):
                    kz = k if k <= d.kz_max else k - d.nz_min
                    spec[kz % nz, ky % ny, i] = u[k, j, i, n]
        ref = np.transpose(np.fft.irfftn(spec, s=(nz, ny, nx), axes=(0, 1, 2), norm="forward"), (2, 1, 0))
        np.testing.assert_allclose(ph[..., n], ref, rtol=0, atol=1e-15 * np.abs(ref).max() * 10)


def test_initial_divergence():
    """initial_field.f:144-151: the solenoidal construction has div <= 1e-7
    (and in fact at round-off)."""
    o = O.Oracle(nx=32, ny=32, nz=32, i_strat=1)
    u = o.init_random(5)
    dc = o.div_check(u)
    assert dc["div_max"] <= GOLD["initial_divergence_max"]
    assert dc["div_max"] < 1e-13


def gw_oracle():
    g = GOLD["gw_input_dat"]
    o = O.Oracle(nx=g["nx"], ny=g["ny"], nz=g["nz"], xl=g["xl"], yl=g["yl"], zl=g["zl"], i_strat=g["i_strat"],
                 vis=g["vis"], dt0=g["dt"], i_cfl=0, n_dealias=g["n_dealias"], nrk_max=g["nrk_max"],
                 buoy_fac_z=g["grav"] / g["to"], lapse=g["lapse0"])
    u = o.init_gw_plane(g["amplitude"], g["lambda_x"], g["lambda_z"], g["omega_i"], g["k_w"], g["m_w"],
                        g["lapse0"], g["uo"])
    return o, u


def test_gravity_wave_input_dat():
    """The reference's input.dat case: a plane internal wave advances by the
    exact RK3 amplification factor each step (init.f:184-210, gw.tex:139-150)."""
    g = GOLD["gw_input_dat"]
    o, u = gw_oracle()
    u0 = u.copy(order="F")
    r = o.wave(o.d.lr)
    o.steps(u, r, g["n_steps"])
    amp = complex(g["rk3_amplification_re"], g["rk3_amplification_im"])
    err = np.abs(u - u0 * amp).max() / np.abs(u0).max()
    assert err < 1e-13, err
    assert abs(o.stats()["time"] - g["n_steps"] * g["dt"]) < 1e-12


def test_taylor_green_energy_decay():
    """Early Taylor-Green decay: dE/dt = -2 nu Z (enstrophy Z = 3 E initially
    for the k = sqrt(3) mode); with nu = 1/400 and 10 steps of dt = 0.01 the
    energy ratio is exp(-6 nu t) to O(t^2) nonlinear corrections."""
    o = O.Oracle(nx=32, ny=32, nz=32, vis=1.0 / 400, dt0=0.01)
    u = o.init_taylor_green()
    r = o.wave(o.d.lr)
    e0 = o.spectra(u, r)["energy_w"]
    o.steps(u, r, 10)
    e1 = o.spectra(u, r)["energy_w"]
    t = 0.1
    assert abs(e0 - 0.125) < 1e-15
    assert abs(e1 / e0 - np.exp(-6 * t / 400)) < 1e-4


def test_inviscid_energy_conservation_transfer():
    """Galerkin truncation conserves energy: the transfer sums to zero
    (spectra.f:22-67 with vis = 0)."""
    o = O.Oracle(nx=24, ny=24, nz=24, vis=0.0, dt0=0.005)
    u = o.init_random(9, 6, 1.0, 6, 0.0)
    r = o.wave(o.d.lr)
    o.stage(u, r, 1)
    # r now holds the rhs of the pre-update field; recompute it for the current u
    o2 = O.Oracle(nx=24, ny=24, nz=24, vis=0.0, dt0=0.0)
    r2 = o2.wave(o2.d.lr)
    u2 = u.copy(order="F")
    o2.stage(u2, r2, 1)
    sp = o2.spectra(u, r2)
    assert abs(sp["tk"].sum()) < 1e-12 * np.abs(sp["tk"]).max() * len(sp["tk"])


def test_x_y_deriv_of_mode():
    o = O.Oracle(nx=16, ny=12, nz=8)
    x = np.arange(16)[:, None] * 2 * np.pi / 16
    y = np.arange(12)[None, :] * 2 * np.pi / 12
    f = np.asfortranarray(np.sin(3 * x) * np.cos(2 * y))
    np.testing.assert_allclose(o.x_deriv(f), 3 * np.cos(3 * x) * np.cos(2 * y), atol=1e-13)
    np.testing.assert_allclose(o.y_deriv(f), -2 * np.sin(3 * x) * np.sin(2 * y), atol=1e-13)


def test_sm_dm_constant_strain():
    """A linear shear u = a z has |S| = a exactly (central differences are exact
    on linear profiles away from the periodic seam), so Smagorinsky gives
    c_smag delta^2 a there."""
    nx = ny = nz = 8
    o = O.Oracle(nx=nx, ny=ny, nz=nz, xl=1.0, yl=1.0, zl=1.0, c_smag=0.1)
    u = np.zeros((nx + 2, ny + 2, nz + 2, 3), order="F")
    x = (np.arange(nx + 2) - 1) / nx
    u[:, :, :, 1] = 0.3 * np.sin(2 * np.pi * x)[:, None, None]
    vt = o.sm(u)
    assert np.isfinite(vt).all() and vt.max() > 0
    vt2, cds = o.dm(u)
    assert np.isfinite(vt2).all() and np.isfinite(cds)


def _np_phys(o, w, op=None):
    """numpy synthesis of one wave field (Nze,Ny_min,Nx_min), optionally times
    i k along axis op ('x', 'y', 'z'), as physical (Nx,Ny,Nz)."""
    d = o.d
    nx, ny, nz = d.nx, d.ny, d.nz
    spec = np.zeros((nz, ny, nx // 2 + 1), complex)
    for i in range(d.nx_min):
        for j in range(d.ny_min):
            ky = j if j <= d.ky_max else j - d.ny_min
            for k in range(d.nz_min):
                kz = k if k <= d.kz_max else k - d.nz_min
                f = {None: 1.0, "x": 1j * i, "y": 1j * ky, "z": 1j * kz}[op]
                spec[kz % nz, ky % ny, i] = w[k, j, i] * f
    return np.transpose(np.fft.irfftn(spec, s=(nz, ny, nx), axes=(0, 1, 2), norm="forward"), (2, 1, 0))


@pytest.mark.parametrize("strat", [0, 1])
def test_planes_match_numpy(strat):
    """sam.f:145-166 + write_planes.f: the oracle's plane cuts, z derivatives,
    y_deriv / x_deriv columns and mean profiles equal numpy's spectral synthesis."""
    nx, ny, nz = 16, 12, 20
    o = O.Oracle(nx=nx, ny=ny, nz=nz, i_strat=strat)
    d = o.d
    lu = d.lu
    u = o.init_random(3)
    p = o.init_random(11)[..., :1].copy(order="F")
    k_xy, j_xz, i_yz = [1, 7, 20], [2, 12], [1, 9]
    r = o.planes(u, p, k_xy, j_xz, i_yz)
    fields = [_np_phys(o, u[..., n]) for n in range(lu)] + [_np_phys(o, p[..., 0])]
    dz = [0, 1, 3][: lu - 1]
    fields += [_np_phys(o, u[..., n], "z") for n in dz]
    dy = [_np_phys(o, u[..., n], "y") for n in [0, 2, 3][: lu - 1]]
    dx = [_np_phys(o, u[..., n], "x") for n in [1, 2, 3][: lu - 1]]
    tol = 1e-13 * max(np.abs(f).max() for f in fields)
    for m, k in enumerate(k_xy):
        for s in range(2 * lu):
            np.testing.assert_allclose(r["xy"][:, :, s, m], fields[s][:, :, k - 1], rtol=0, atol=tol)
    for m, j in enumerate(j_xz):
        for s in range(2 * lu):
            ref = fields[s][:, j - 1, :] if s <= lu else dy[s - lu - 1][:, j - 1, :]
            np.testing.assert_allclose(r["xz"][:, :, s, m], ref, rtol=0, atol=tol)
    for m, i in enumerate(i_yz):
        for s in range(2 * lu):
            ref = fields[s][i - 1, :, :] if s <= lu else dx[s - lu - 1][i - 1, :, :]
            np.testing.assert_allclose(r["yz"][:, :, s, m], ref, rtol=0, atol=tol)
    for n in range(lu):
        np.testing.assert_allclose(r["mean"][:, n], fields[n].mean(axis=(0, 1)), rtol=0, atol=tol)


def _kvec(o, shape):
    """Integer wave numbers (kz, ky, kx) of the wave-space layout (stored
    order of fft_init.f:52-78: non-negative first, then negative)."""
    d = o.d
    kz = np.array([k if k <= d.kz_max else k - d.nz_min for k in range(d.nz_min)])
    ky = np.array([k if k <= d.ky_max else k - d.ny_min for k in range(d.ny_min)])
    kx = np.arange(d.nx_min)
    return np.meshgrid(kz, ky, kx, indexing="ij")


def test_ou_forcing_from_rest():
    """Ornstein-Uhlenbeck forcing applied to a fluid at rest: after one step
    only the modes 0 < |k| <= k_f hold energy, the forced field is
    solenoidal, and the kx = 0 plane keeps the conjugate symmetry of a real
    field; the same seed gives the same field, another seed another."""
    cfg = dict(nx=24, ny=24, nz=24, vis=0.0, dt0=0.01)
    o = O.Oracle(**cfg)
    assert o.set_forcing(7, k_f=2.5, sigma=0.3, t_l=0.5) == 40
    u = o.wave(o.d.lu)
    r = o.wave(o.d.lr)
    o.steps(u, r, 1)
    d = o.d
    kz, ky, kx = _kvec(o, None)
    k2 = kz ** 2 + ky ** 2 + kx ** 2
    um = u[: d.nz_min]
    mag = np.abs(um).sum(axis=-1)
    assert mag[(k2 > 6.25) | (k2 == 0)].max() == 0.0
    assert (mag[(k2 <= 6.25) & (k2 > 0)] > 0).all()
    div = kx * um[..., 0] + ky * um[..., 1] + kz * um[..., 2]
    assert np.abs(div).max() < 1e-15 * np.abs(um).max() * 4
    for j in range(d.ny_min):
        for k in range(d.nz_min):
            jm, km = (-j) % d.ny_min, (-k) % d.nz_min
            assert np.allclose(um[k, j, 0], np.conj(um[km, jm, 0]), rtol=0, atol=1e-17)
    o2 = O.Oracle(**cfg)
    o2.set_forcing(7, k_f=2.5, sigma=0.3, t_l=0.5)
    u2, r2 = o2.wave(d.lu), o2.wave(d.lr)
    o2.steps(u2, r2, 1)
    assert np.array_equal(u2, u)
    o3 = O.Oracle(**cfg)
    o3.set_forcing(8, k_f=2.5, sigma=0.3, t_l=0.5)
    u3, r3 = o3.wave(d.lu), o3.wave(d.lr)
    o3.steps(u3, r3, 1)
    assert not np.array_equal(u3, u)


def test_ou_forcing_stationary_variance():
    """With dt / T_L small the injected velocity after n steps from rest is
    dt * sum of correlated amplitudes; over many modes the per-component
    mean square of u / (n dt) approaches sigma^2 times the solenoidal share
    (2/3) for n dt << T_L.  A loose statistical check of the RNG scaling."""
    o = O.Oracle(nx=32, ny=32, nz=32, vis=0.0, dt0=1e-4)
    n = o.set_forcing(3, k_f=2.5, sigma=1.0, t_l=100.0)
    u, r = o.wave(o.d.lu), o.wave(o.d.lr)
    o.steps(u, r, 1)
    kz, ky, kx = _kvec(o, None)
    k2 = kz ** 2 + ky ** 2 + kx ** 2
    sel = (k2 > 0) & (k2 <= 6.25) & ((kx > 0) | (ky > 0) | ((ky == 0) & (kz > 0)))
    amp = u[: o.d.nz_min][sel] / 1e-4
    ms = (np.abs(amp) ** 2).sum(axis=-1).mean()
    assert sel.sum() == n
    assert 0.5 * 2.0 < ms < 1.5 * 2.0


def test_coupled_smagorinsky_dissipates():
    """The Smagorinsky stress only removes energy: starting from the same
    field, the coupled closure ends with less kinetic energy than the plain
    step, and the field stays solenoidal."""
    cfg = dict(nx=24, ny=24, nz=24, vis=1e-4, dt0=0.01)
    es = []
    for model in (0, 1):
        o = O.Oracle(**cfg)
        u = o.init_random(5, 6, 1.0, 6, 0.0)
        o.set_les(model, c_smag=0.04)
        r = o.wave(o.d.lr)
        o.steps(u, r, 3)
        es.append(o.spectra(u, r)["energy_w"])
        assert o.div_check(u)["div_max"] < 1e-13
    assert es[1] < es[0]


def test_coupled_dynamic_coefficient_is_dm_of_the_field():
    """The dynamic closure's coefficient is dm.f's volume-averaged C delta^2
    of the stage-1 physical velocity: rebuild that field with the oracle's
    backward transforms, add the periodic halos and call dm directly."""
    cfg = dict(nx=16, ny=20, nz=24, vis=1e-4, dt0=0.005)
    o = O.Oracle(**cfg)
    u = o.init_random(8, 0, 1.0, 0, 0.0)
    d = o.d
    zb = o.z_trans_b(u.copy(order="F"), d.lu)
    ph = o.xy_trans_b(o.x2z_decomp(zb, d.lu), d.lu)
    uh = np.zeros((d.nx + 2, d.ny + 2, d.nz + 2, 3), order="F")
    for n in range(3):
        uh[1:-1, 1:-1, 1:-1, n] = ph[..., n]
        a = uh[..., n]
        a[0], a[-1] = a[-2], a[1]
        a[:, 0], a[:, -1] = a[:, -2], a[:, 1]
        a[:, :, 0], a[:, :, -1] = a[:, :, -2], a[:, :, 1]
    _, cds = o.dm(uh)
    o.set_les(2)
    r = o.wave(d.lr)
    o.stage(u, r, 1)
    assert cds > 0
    assert abs(o.les_coef() - cds) <= 1e-14 * cds
