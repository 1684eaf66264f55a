"""Training data, training and evaluation of the learned subgrid closure.

The reference has no learned model: its subgrid routines are sm.f and dm.f,
and this module makes the data the network learns from with the solver
itself, on the GPU:

1. a DNS on a fine grid (stratified Boussinesq, seeded random start, low
   wavenumber Ornstein-Uhlenbeck forcing) advanced by sam_gpu_step;
2. snapshots box-filtered and downsampled by f on the GPU
   (sam_gpu_box_filter): block means of u_a, T, u_a u_b and u_a T;
3. the filtered velocity and temperature taken to the coarse grid's wave
   space with the reference's forward transforms (xy_trans_f, z_trans_f) in a
   coarse context, projected on divergence-free modes, and uploaded;
4. the closure's invariants and the resolved gradients on the coarse grid
   (sam_gpu_closure_inputs);
5. targets from the exact subgrid fluxes of the filter,
      tau_ab = <u_a u_b> - <u_a><u_b>,   q_a = <u_a T> - <u_a><T>,
      nu*    = -tau^d_ab S_ab / (2 S_ab S_ab),   C_nu*    = nu* / (delta^2 |S|),
      kappa* = -q_a dT/dx_a / |grad T|^2,        C_kappa* = kappa* / (delta^2 |S|),
   clipped to [0, C_MAX] (the network's coefficients are non-negative);
6. training with Adam on the device (sam_gpu_mlp_train).

evaluate_a_priori compares the trained network, dm.f's dynamic coefficient
and the no-model case on held-out data; evaluate_a_posteriori runs coarse
LES from a filtered snapshot with each closure and compares kinetic-energy
spectra with the filtered DNS.
"""
from __future__ import annotations

import math
import os

import numpy as np

from .sam_gpu import MLP_FEATURES, MLP_PARAMS, SamGpu

C_MAX = 0.1
HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "data", "closure_mlp.npz")


def dns_config(n, precision=32, vis=1e-3):
    """Stratified turbulence, N = 1 (buoy_fac_z = lapse = 1), Pr = 1, CFL 0.5."""
    return dict(nx=n, ny=n, nz=n, i_strat=1, i_cfl=1, cfl0=0.5, vis=vis, pr=1.0, dt0=1e-3, buoy_fac_z=1.0,
                lapse=1.0, precision=precision)


def coarse_config(n, vis=1e-3, precision=64):
    return dict(dns_config(n, precision, vis))


def advance_to(g, t_end, chunk=20):
    while g.stats()["time"] < t_end:
        g.step(chunk)
        st = g.stats()
        if st["nonfinite"]:
            raise FloatingPointError("DNS blew up (non-finite velocity)")


def dns_snapshots(n=512, filters=(4,), n_snap=10, t_spinup=1.0, t_every=0.1, seed=0, vis=1e-3, precision=32,
                  forcing=(2.5, 0.5, 0.5), t_eval=0.2, n_eval=1, log=print):
    """Filtered snapshots (X, Y, Z, Lu+Lr) of a forced stratified DNS for
    every filter ratio f in `filters` ({f: [snapshots]}), and an evaluation
    sequence: after the training snapshots the forcing stops and the
    filtered field is taken at t0 and at n_eval later times spaced
    t_eval / n_eval apart (decaying, so a coarse LES can follow it without
    the DNS's random forcing): {f: [fields]} and the times after t0."""
    g = SamGpu(**dns_config(n, precision, vis))
    try:
        g.init_random(seed, 6, 1.0, 6, 0.1)
        if forcing:
            g.set_forcing(seed + 1, *forcing)
        advance_to(g, t_spinup)
        snaps = {f: [] for f in filters}
        for s in range(n_snap):
            for f in filters:
                snaps[f].append(g.box_filter(f))
            st = g.stats()
            log(f"snapshot {s}: t = {st['time']:.3f}, energy {st['energy']:.4f}, u_max {st['u_max'][:3]}")
            advance_to(g, st["time"] + t_every)
        g.set_forcing(0, 0.0)
        ev = {f: [g.box_filter(f)] for f in filters}
        t0 = g.stats()["time"]
        times = []
        for e in range(n_eval):
            advance_to(g, t0 + t_eval * (e + 1) / n_eval, chunk=1)
            times.append(g.stats()["time"] - t0)
            for f in filters:
                ev[f].append(g.box_filter(f))
        log(f"evaluation sequence: t = {t0:.3f} + {times}")
        return snaps, (ev, times)
    finally:
        g.close()


def to_wave(g, phys):
    """Physical (X, Y, Z, Lu) -> the coarse wave layout (Nze, Ny_min, Nx_min, Lu),
    projected on divergence-free modes (the filter does not keep the field
    exactly solenoidal on the coarse grid)."""
    lu = phys.shape[-1]
    w = g.xy_trans_f(np.asfortranarray(phys.copy()), lu)
    w = g.z_trans_f(w, lu)
    kx = np.arange(g.nx_min)
    ky = np.array([j if j <= g.ky_max else j - g.ny_min for j in range(g.ny_min)])
    kz = np.array([k if k <= g.kz_max else k - g.nz_min for k in range(g.nz_min)] + [0] * (g.nze - g.nz_min))
    KZ, KY, KX = np.meshgrid(kz, ky, kx, indexing="ij")
    k2 = np.maximum(KX ** 2 + KY ** 2 + KZ ** 2, 1e-30)
    div = (KX * w[..., 0] + KY * w[..., 1] + KZ * w[..., 2]) / k2
    w[..., 0] -= KX * div
    w[..., 1] -= KY * div
    w[..., 2] -= KZ * div
    w[g.nz_min:] = 0
    return np.asfortranarray(w)


def targets(filt, grads, lu, dsq):
    """(C_nu*, C_kappa*) per coarse point from the filtered fields and the
    coarse resolved gradients (Fortran-ordered (X, Y, Z, .) arrays)."""
    ub = [filt[..., a] for a in range(3)]
    pairs = [(0, 0), (0, 1), (1, 1), (0, 2), (1, 2), (2, 2)]
    tau = [filt[..., lu + m] - ub[a] * ub[b] for m, (a, b) in enumerate(pairs)]
    tr = (tau[0] + tau[2] + tau[5]) / 3.0
    tau[0] = tau[0] - tr
    tau[2] = tau[2] - tr
    tau[5] = tau[5] - tr
    wts = [1, 2, 1, 2, 2, 1]
    S = [grads[..., m] for m in range(6)]
    ss = sum(w * s * s for w, s in zip(wts, S))
    ts = sum(w * t * s for w, t, s in zip(wts, tau, S))
    smag = np.sqrt(2 * ss)
    with np.errstate(divide="ignore", invalid="ignore"):
        nu = -ts / (2 * ss)
        cnu = np.where(ss > 0, nu / (dsq * smag), 0.0)
    if lu == 4:
        tb = filt[..., 3]
        q = [filt[..., lu + 6 + a] - ub[a] * tb for a in range(3)]
        gT = [grads[..., 6 + a] for a in range(3)]
        g2 = sum(x * x for x in gT)
        with np.errstate(divide="ignore", invalid="ignore"):
            kap = -sum(qa * ga for qa, ga in zip(q, gT)) / g2
            ck = np.where((g2 > 0) & (ss > 0), kap / (dsq * smag), 0.0)
    else:
        ck = np.zeros_like(cnu)
    raw = np.stack([cnu.ravel(order="F"), ck.ravel(order="F")], axis=1)
    return np.clip(np.nan_to_num(raw), 0.0, C_MAX).astype(np.float32), raw, smag.ravel(order="F")


def coarse_samples(snaps, n_coarse, vis=1e-3):
    """Features [N][12], targets [N][2] (and the unclipped targets, |S|) of
    every coarse point of every snapshot."""
    g = SamGpu(**coarse_config(n_coarse, vis))
    try:
        lu = g.lu
        dx = 2 * math.pi / n_coarse
        dsq = (dx ** 3) ** (2.0 / 3.0)
        F, Y, R, SM = [], [], [], []
        for filt in snaps:
            g.upload(to_wave(g, filt[..., :lu]))
            feat, grads = g.closure_inputs()
            # closure_inputs orders points (z Ny + y) Nx + x, i.e. Fortran order of (X, Y, Z)
            y, raw, smag = targets(filt, grads, lu, dsq)
            F.append(feat)
            Y.append(y)
            R.append(raw)
            SM.append(smag)
        return np.concatenate(F), np.concatenate(Y), np.concatenate(R), np.concatenate(SM), dsq
    finally:
        g.close()


def train(features, target, steps=None, batch=8192, lr=1e-3, seed=0, init=None, n_coarse=16):
    """Shuffle, then Adam on the device; returns (params, loss history)."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(len(features))
    x, y = features[perm], target[perm]
    steps = steps or max(1, len(x) // batch)
    if init is None:
        init = init_params(seed)
    g = SamGpu(nx=n_coarse, ny=n_coarse, nz=n_coarse)
    try:
        g.mlp_set(init)
        hist = g.mlp_train(x, y, steps, batch, lr)
        return g.mlp_get(), hist
    finally:
        g.close()


def init_params(seed=0):
    """He-style initial weights, zero biases, a small last layer."""
    rng = np.random.default_rng(seed)
    nh, ni, no = 64, MLP_FEATURES, 2
    p = np.zeros(MLP_PARAMS, dtype=np.float32)
    o = 0
    p[o:o + nh * ni] = rng.standard_normal(nh * ni) * np.sqrt(2.0 / ni)
    o += nh * ni + nh
    p[o:o + nh * nh] = rng.standard_normal(nh * nh) * np.sqrt(2.0 / nh)
    o += nh * nh + nh
    p[o:o + no * nh] = rng.standard_normal(no * nh) * 0.1 / np.sqrt(nh)
    return p


def predict(params, features, n_coarse=16):
    g = SamGpu(nx=n_coarse, ny=n_coarse, nz=n_coarse)
    try:
        g.mlp_set(params)
        return g.mlp_forward(features)
    finally:
        g.close()


def _corr(a, b):
    a = a - a.mean()
    b = b - b.mean()
    return float((a * b).sum() / np.sqrt((a * a).sum() * (b * b).sum() + 1e-300))


def dm_coefficient(filt, n_coarse, vis=1e-3):
    """dm.f's volume-averaged C delta^2 of a filtered snapshot on the coarse
    grid (the coefficient the dynamic closure would use there)."""
    g = SamGpu(**coarse_config(n_coarse, vis))
    try:
        g.upload(to_wave(g, filt[..., :g.lu]))
        g.set_les(2)
        g.stage(1)
        return g.les_coef()
    finally:
        g.close()


def evaluate_a_priori(params, feat, raw, smag, dsq, c_dm):
    """Correlation with the exact nu*, and the mean subgrid dissipation
    <nu_t |S|^2> relative to the exact <nu* |S|^2>, for the network, for
    dm.f's dynamic coefficient (a constant C, so its correlation is that of
    |S| alone) and for no model."""
    nu_true = raw[:, 0] * dsq * smag
    c = predict(params, feat)
    nu_net = c[:, 0] * dsq * smag
    nu_dm = max(c_dm, 0.0) * smag
    eps = lambda nu: float((nu * smag ** 2).mean())  # noqa: E731
    e_true = eps(nu_true)
    return {
        "corr_net": _corr(nu_net, nu_true), "corr_dm": _corr(nu_dm, nu_true),
        "dissipation_net": eps(nu_net) / e_true, "dissipation_dm": eps(nu_dm) / e_true, "dissipation_none": 0.0,
        "c_dm_over_delta_sq": c_dm / dsq, "mean_c_net": float(c[:, 0].mean()),
    }


def shell_spectrum(g):
    return g.spectra()["ek"]


def evaluate_a_posteriori(params, fields, times, n_coarse, vis=1e-3, kmax_frac=0.5):
    """Coarse LES from the filtered snapshot fields[0] with no model, dm.f's
    dynamic closure and the learned closure, compared with the filtered DNS
    fields[1:] at the elapsed times `times`: per closure the relative
    spectrum error over shells k <= kmax_frac * k_max (the largest over the
    shells, averaged over the comparison times), the same over all shells
    k <= k_max, and the spectra at the last time."""
    g = SamGpu(**coarse_config(n_coarse, vis))
    try:
        refs = []
        for fld in fields[1:]:
            g.upload(to_wave(g, fld[..., :g.lu]))
            refs.append(shell_spectrum(g))
        u0 = to_wave(g, fields[0][..., :g.lu])
        kmax = int((n_coarse - 0.1) / 3)
        ks = np.arange(1, int(kmax_frac * kmax) + 1)
        ka = np.arange(1, kmax + 1)
        out = {"times": list(times)}
        for name, model in (("none", 0), ("dm", 2), ("net", 3)):
            g.upload(u0)
            g.set_tstep(1, 1e-3, 0.0)
            if model == 3:
                g.mlp_set(params)
            g.set_les(model)
            e_half, e_all = [], []
            for t, ref in zip(times, refs):
                advance_to(g, t, chunk=5)
                ek = shell_spectrum(g)
                e_half.append(float(np.abs(ek[ks] / ref[ks] - 1).max()))
                e_all.append(float(np.abs(ek[ka] / ref[ka] - 1).max()))
            g.set_les(0)
            out[name] = float(np.mean(e_half))
            out[f"{name}_all_shells"] = float(np.mean(e_all))
            out[f"spectrum_{name}"] = ek[: kmax + 1].tolist()
        out["spectrum_dns"] = refs[-1][: kmax + 1].tolist()
        return out
    finally:
        g.close()


def run(n=512, filters=(4,), n_snap=10, steps=None, batch=8192, lr=1e-3, vis=1e-3, t_spinup=1.0, t_every=0.1,
        t_eval=0.2, n_eval=1, seed=0, out=WEIGHTS, log=print, forcing=(2.5, 0.5, 0.5)):
    """The whole pipeline: DNS snapshots filtered at every ratio in
    `filters`, samples, one network trained on all of them but the last
    snapshot, a priori evaluation on that one and a posteriori evaluation on
    the decaying sequence, per filter ratio; saves the parameters and the
    report."""
    import json
    import time

    t0 = time.time()
    snaps, (ev, times) = dns_snapshots(n, filters, n_snap, t_spinup, t_every, seed, vis, forcing=forcing,
                                       t_eval=t_eval, n_eval=n_eval, log=log)
    t1 = time.time()
    data = {}
    for f in filters:
        nc = n // f
        feat, y, raw, smag, dsq = coarse_samples(snaps[f], nc, vis)
        npt = nc ** 3
        data[f] = dict(nc=nc, feat=feat, y=y, raw=raw, smag=smag, dsq=dsq, tr=slice(0, npt * (n_snap - 1)),
                       te=slice(npt * (n_snap - 1), npt * n_snap))
    x_tr = np.concatenate([d["feat"][d["tr"]] for d in data.values()])
    y_tr = np.concatenate([d["y"][d["tr"]] for d in data.values()])
    t2 = time.time()
    params, hist = train(x_tr, y_tr, steps, batch, lr, seed)
    t3 = time.time()
    per_filter = {}
    for f, d in data.items():
        te, tr = d["te"], d["tr"]
        c_dm = dm_coefficient(snaps[f][-1], d["nc"], vis)
        prior = evaluate_a_priori(params, d["feat"][te], d["raw"][te], d["smag"][te], d["dsq"], c_dm)
        c_test = predict(params, d["feat"][te])
        prior["mse_net"] = float(((c_test - d["y"][te]) ** 2).mean())
        prior["mse_mean"] = float(((d["y"][tr].mean(0) - d["y"][te]) ** 2).mean())
        post = evaluate_a_posteriori(params, ev[f], times, d["nc"], vis)
        per_filter[str(f)] = {
            "coarse": d["nc"], "a_priori": prior,
            "a_posteriori_max_rel_err_k_le_kmax_half": {k: post[k] for k in ("none", "dm", "net")},
            "a_posteriori_max_rel_err_all_shells": {k: post[f"{k}_all_shells"] for k in ("none", "dm", "net")},
            "a_posteriori_times": post["times"],
            "spectra": {k: post[k] for k in post if k.startswith("spectrum")}}
    report = {"dns": n, "filters": list(filters), "snapshots": n_snap, "samples_train": int(len(x_tr)),
              "forcing": list(forcing), "vis": vis, "steps": int(len(hist)), "batch": batch, "lr": lr,
              "loss_first": float(hist[:10].mean()), "loss_last": float(hist[-10:].mean()),
              "per_filter": {f: {k: v for k, v in r.items() if k != "spectra"} for f, r in per_filter.items()},
              "seconds": {"dns": t1 - t0, "samples": t2 - t1, "train": t3 - t2}}
    # the first filter's figures at the top level as well (the layout the
    # single-filter report had)
    first = per_filter[str(filters[0])]
    report.update({"filter": filters[0], "coarse": first["coarse"], "a_priori": first["a_priori"],
                   "a_posteriori_max_rel_err_k_le_kmax_half": first["a_posteriori_max_rel_err_k_le_kmax_half"]})
    log(json.dumps(report))
    if out:
        os.makedirs(os.path.dirname(out), exist_ok=True)
        np.savez(out, params=params, loss=hist, report=json.dumps(report),
                 spectra=json.dumps({f: r["spectra"] for f, r in per_filter.items()}))
    return params, report


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description="train the learned closure on filtered DNS")
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--filters", type=int, nargs="+", default=[4, 8], help="box-filter ratios of the samples")
    ap.add_argument("--snaps", type=int, default=10)
    ap.add_argument("--steps", type=int, default=12000, help="Adam steps (0: one pass over the data)")
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--vis", type=float, default=5e-4)
    ap.add_argument("--spinup", type=float, default=1.0)
    ap.add_argument("--every", type=float, default=0.1)
    ap.add_argument("--eval", type=float, default=1.0, help="a posteriori comparison window")
    ap.add_argument("--neval", type=int, default=4, help="comparison times in the window")
    ap.add_argument("--sigma", type=float, default=0.15, help="OU forcing rms amplitude")
    ap.add_argument("--tl", type=float, default=0.5, help="OU forcing correlation time")
    ap.add_argument("--out", default=WEIGHTS)
    a = ap.parse_args()
    run(a.n, tuple(a.filters), a.snaps, a.steps or None, a.batch, a.lr, a.vis, a.spinup, a.every, a.eval, a.neval,
        out=a.out, forcing=(2.5, a.sigma, a.tl))
