#!/usr/bin/env python
"""Benchmark: RK3 steps/s of the SAM pseudo-spectral step on one GB300.

Workload (the 256^3 configuration the headline metric is quoted on): the
internal-gravity-wave packet in a 256^3 periodic [0, 2pi]^3 box, Boussinesq
with N = 2 (buoy_fac_z * lapse = 4), nu = kappa = 1e-4, Gaussian-enveloped
plane wave k = (8, 0, 16), envelope width pi/4, amplitude 0.05, plus a seeded
1 % white-noise velocity; RK3 with dt from the CFL number 0.5 (vel_max every
step).  Synthetic seeded input, generated on the device.

  value : FP64 drop-in steps/s with the state resident in HBM (CUDA graph of
          a whole step), timed with CUDA events on the launching stream.
  e2e   : the same metric through the C ABI with host buffers: each step
          uploads u from pinned host memory, runs the step, downloads u.
  fp32  : the FP32-bulk form (FP64 reductions) on the same workload, with its
          relative error against the FP64 run after the timed steps.
  les   : LES of stratified forced turbulence at 256^3 (N = 1, OU forcing of
          |k| <= 2.5): the FP64 drop-in with dm.f's dynamic Smagorinsky
          coupled in against the FP32 bulk form with the learned closure
          (tcgen05 network), steps/s of each, their ratio, and the spectrum
          difference for k <= k_max/2 after the timed steps.
  ensemble: 96 independent members of uneven sizes in one graph per step
          (aggregate member-steps/s) against the members run one by one in
          the plain FP64 drop-in.

`--impl reference` times the reference algorithm on the host cores instead
(the oracle, a C restatement of the Fortran path; the Fortran reference itself
cannot be built: no Fortran compiler or MPI on this machine).

Multi-GPU (`--gpus N` under torchrun): independent replicas, one per GPU, no
data-path collective; value = total steps of all replicas / max time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 256
WORKLOAD = ("gravity-wave packet 256^3 stratified Boussinesq, N=2, nu=kappa=1e-4, k0=(8,0,16), "
            "width pi/4, amplitude 0.05, 1% noise, RK3 CFL 0.5")
METRIC = ("RK3 steps/s at 256^3 (FP64 drop-in; FP32 bulk, FP64 + dm.f LES and FP32 + learned-closure LES "
          "reported beside it)")


def workload_cfg(n=None, precision=64):
    n = n or N
    return dict(nx=n, ny=n, nz=n, i_strat=1, i_cfl=1, cfl0=0.5, vis=1e-4, pr=1.0, dt0=1e-3,
                buoy_fac_z=4.0, lapse=1.0, precision=precision)


PACKET = dict(seed=1, k0=(8, 0, 16), sigma=math.pi / 4, amplitude=0.05, noise=0.01)


def dims(n=None, lu=4, lr=9):
    n = n or N
    k = int((n - 0.1) / 3.0)
    mx, my, mz = k + 1, 2 * k + 1, 2 * k + 1
    return mx, my, mz


def algorithmic_bytes_per_step(n=None, w=8, lu=4, lr=9):
    """Bytes one stage must move with the transposes fused into the passes:
    z inverse, y inverse, x pass (C2R, products, R2C), y forward, z forward
    with the update (read u, r_old; write u, r, p); three stages per step."""
    n = n or N
    mx, my, mz = dims(n)
    sz, szn, syn = mx * my * mz, mx * my * n, mx * n * n
    c = 2 * w
    stage = c * (lu * (sz + szn) + lu * (szn + syn) + (lu + lr) * syn + lr * (syn + szn) + lr * szn
                 + 4 * lu * sz + sz)
    return 3 * stage


def x_pass_bytes(n=None, w=8, lu=4, lr=9):
    n = n or N
    mx, _, _ = dims(n)
    return 2 * w * (lu + lr) * mx * n * n


def x_pass_flops(n=None, lu=4, lr=9):
    n = n or N
    # 5 n log2 n per complex line; two real x-lines share one complex line
    return 5.0 * n * math.log2(n) * (lu + lr) * n * (n / 2)


def step_flops(n=None, lu=4, lr=9):
    n = n or N
    mx, my, _ = dims(n)
    f = 5.0 * n * math.log2(n)
    per_field = mx * my * f + mx * n * f + n * n * f / 2
    return 3 * (lu + lr) * per_field


class Clocks:
    """nvidia-smi samples during the timed region (SM clock, reasons)."""

    def __init__(self, gpu_index=0):
        self.samples, self.proc, self.idx = [], None, gpu_index

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx = max(mx, float(s[1]))
                for nm, v in zip(names, s[3:7]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def profile_traffic(name="x_pass_traffic.json"):
    """DRAM traffic per x-pass launch from the committed ncu summary, if any;
    the summaries cover the 256^3 workload, so other grids get none."""
    if N != 256:
        return None
    try:
        return json.load(open(os.path.join(ROOT, "profiles", name)))
    except (OSError, ValueError):
        return None


def max_over_ranks(x, pg):
    """The largest value of x over the ranks of pg (x itself with one rank):
    the timed region of the job is the slowest replica's."""
    if not pg:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t[0])


def whole_job_rate(steps, seconds, ws):
    """Steps per second of the whole job: ws replicas each ran `steps` steps
    (weak scaling) in `seconds`, the slowest rank's time."""
    return ws * steps / seconds


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")), ws


def cpu_oracle_rate(n, steps, threads, warm_stages=1, u_start=None):
    """Steps/s of the oracle (C restatement of the reference path, OpenMP)
    over `steps` steps from the workload's start (or u_start); also returns
    the state after them.  The warm-up stages run on a copy."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    cfg = workload_cfg(n)
    cfg.pop("precision")
    o = O.Oracle(nthreads=threads, **cfg)
    if u_start is None:
        u = o.init_packet(PACKET["seed"], PACKET["k0"], PACKET["sigma"], PACKET["amplitude"], PACKET["noise"])
    else:
        u = u_start.copy(order="F")
    uw, rw = u.copy(order="F"), o.wave(o.d.lr)
    for s in range(warm_stages):
        o.stage(uw, rw, 1)
    o.close()
    o = O.Oracle(nthreads=threads, **cfg)
    r = o.wave(o.d.lr)
    t0 = time.perf_counter()
    o.steps(u, r, steps)
    dt = time.perf_counter() - t0
    st = o.stats()
    nz_min = o.d.nz_min
    o.close()
    return steps / dt, dt, u, st, nz_min


def parity_vs_oracle(u_start, u_oracle, st_oracle, nz_min, steps, stream):
    """The same `steps` steps on the GPU from u_start (FP64 drop-in and FP32
    bulk, fresh contexts) against the oracle's state: the largest error per
    field relative to the field's largest coefficient, the CFL dt and the
    divergence of the result."""
    import numpy as np
    from sam_gb300 import SamGpu
    out = {"steps": steps, "bar_fp64": 1e-12,
           "measure": "max |u_gpu - u_oracle| / max |u_oracle| per field (Nz_min rows)"}
    for name, prec in (("fp64", 64), ("double_float", 48), ("fp32_bulk", 32)):
        g = SamGpu(**workload_cfg(precision=prec))
        g.set_stream(stream.cuda_stream)
        g.upload(u_start)
        g.step(steps)
        ug = g.download()
        err = [float(np.abs(ug[:nz_min, ..., n] - u_oracle[:nz_min, ..., n]).max()
                     / np.abs(u_oracle[:nz_min, ..., n]).max()) for n in range(u_oracle.shape[-1])]
        st = g.stats()
        out[name] = {"max_rel_err_per_field": err, "dt_rel_diff": abs(st["dt"] - st_oracle["dt"]) / st_oracle["dt"],
                     "div_max": g.div_check()["div_max"]}
        g.close()
    out["fp64_within_bar"] = max(out["fp64"]["max_rel_err_per_field"]) <= 1e-12
    out["double_float_within_bar"] = max(out["double_float"]["max_rel_err_per_field"]) <= 1e-12
    return out


def band_errors(u, ref):
    """Relative L2 error of u against ref per field and per spectral band of
    the shell index |k| (wave numbers of the 2 pi box): [1, K/4), [K/4, K/2),
    [K/2, sqrt(3) K] with K = k_max (arrays in the wave layout, Nze rows)."""
    import numpy as np
    mx, my, mz = dims()
    k = (mx - 1)
    kx = np.arange(mx)
    ky = np.array([j if j <= k else j - my for j in range(my)])
    kz = np.array([q if q <= k else q - mz for q in range(mz)])
    KZ, KY, KX = np.meshgrid(kz, ky, kx, indexing="ij")
    shell = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    w = np.where(KX == 0, 1.0, 2.0)  # conjugate modes of kx > 0
    edges = [(1, k / 4), (k / 4, k / 2), (k / 2, np.sqrt(3) * k + 1)]
    out = {}
    for n in range(u.shape[-1]):
        d, r = u[:mz, ..., n], ref[:mz, ..., n]
        row = {}
        for lo, hi in edges:
            sel = (shell >= lo) & (shell < hi)
            num = float((w[sel] * np.abs(d[sel] - r[sel]) ** 2).sum())
            den = float((w[sel] * np.abs(r[sel]) ** 2).sum())
            row[f"k{lo:.0f}-{hi:.0f}"] = (num / den) ** 0.5 if den > 0 else None
        out[f"field{n}"] = row
    return out


def closure_params():
    """The trained closure network (sam_gb300/data/closure_mlp.npz, made by
    python -m sam_gb300.closure_data on the GPU) or, without it, the
    untrained initial network (the timing does not depend on the weights)."""
    import numpy as np
    from sam_gb300 import closure_data as CD
    try:
        z = np.load(CD.WEIGHTS)
        return z["params"], "trained (" + os.path.relpath(CD.WEIGHTS, ROOT) + ")"
    except (OSError, KeyError):
        return CD.init_params(0), "untrained initial weights"


LES_WORKLOAD = ("LES of stratified forced turbulence 256^3, N=1 (buoy_fac_z = lapse = 1), Pr=1, nu=1e-4, "
                "random solenoidal start k^4 exp(-2(k/4)^2) at rms 1 (seed 3), T at 0.1, OU forcing of "
                "|k| <= 2.5 (sigma 0.15, T_L 0.5, seed 4), RK3 CFL 0.5")


def les_cfg(precision):
    return dict(nx=N, ny=N, nz=N, i_strat=1, i_cfl=1, cfl0=0.5, vis=1e-4, pr=1.0, dt0=1e-3, buoy_fac_z=1.0,
                lapse=1.0, precision=precision)


def les_forms(stream, K, W, t_spin=1.5, t_win=6.0, n_win=30):
    """The LES workload.  Speed: the FP64 drop-in with dm.f's dynamic closure
    and the FP32 bulk form with the learned closure, K steps each from their
    developed state after W warm-up steps (CUDA events on the launching
    stream).  Spectra: dm.f's dynamic closure, the learned closure and no
    model (a control), each in the FP32 bulk form and spun up on its own from
    the same random start and OU forcing to t_spin, the kinetic-energy
    spectrum averaged over n_win samples of the window (t_spin, t_spin +
    t_win] (long, so that the forced low shells' fluctuations average out),
    and the largest relative difference from the dm.f run's over shells
    k <= k_max/2."""
    import numpy as np
    import torch
    from sam_gb300 import SamGpu
    params, src = closure_params()
    out = {"workload": LES_WORKLOAD,
           "comparison": f"FP32 forms, each spun up independently from the same start to t = {t_spin}, E(k) "
                         f"averaged over {n_win} samples in t in ({t_spin}, {t_spin + t_win}]"}

    def advance(g, t_end, chunk=10):
        while g.stats()["time"] < t_end:
            g.step(chunk)

    def start(prec, model):
        g = SamGpu(**les_cfg(prec))
        g.set_stream(stream.cuda_stream)
        g.init_random(3, 6, 1.0, 6, 0.1)
        g.set_forcing(4, 2.5, 0.15, 0.5)
        if model == 3:
            g.mlp_set(params)
        if model:
            g.set_les(model)
        g.autotune(3)  # tiles for this form's passes (setup, outside the timed region)
        return g

    def timed(g):
        g.step(W)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            g.step(K)
            e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        passes = [g.profile_stage(nrk, 2) for nrk in (1, 2, 3)]
        return {"value": K / (ms / 1e3), "unit": "steps/s", "ms_per_step": ms / K,
                "passes_ms": {k: sum(p[k] for p in passes) / 3 for k in passes[0]}}

    # speed of the FP64 + dm.f drop-in (developed over half a time unit)
    g = start(64, 2)
    advance(g, 0.5)
    out["fp64_dm"] = timed(g)
    out["fp64_dm"]["c_delta_sq_final"] = g.les_coef()
    g.close()
    avg = {}
    for name, model in (("fp32_dm", 2), ("fp32_learned", 3), ("fp32_none", 0)):
        g = start(32, model)
        advance(g, 0.5)
        row = timed(g) if model == 3 else {}
        advance(g, t_spin)
        eks = []
        for i in range(n_win):
            advance(g, t_spin + t_win * (i + 1) / n_win)
            eks.append(g.spectra()["ek"])
        avg[name] = np.mean(eks, axis=0)
        st = g.stats()
        row.update({"time_final": st["time"], "energy_final": st["energy"]})
        out[name] = row
        g.close()
    kmax = int((N - 0.1) / 3)
    ks = np.arange(1, kmax // 2 + 1)
    out["speedup_fp32_learned_over_fp64_dm"] = out["fp32_learned"]["value"] / out["fp64_dm"]["value"]
    out["spectrum_max_rel_diff_k_le_kmax_half"] = float(np.abs(avg["fp32_learned"][ks] / avg["fp32_dm"][ks] - 1).max())
    out["spectrum_max_rel_diff_k_le_kmax_half_no_model"] = float(
        np.abs(avg["fp32_none"][ks] / avg["fp32_dm"][ks] - 1).max())
    out["spectrum_rel_diff_per_shell_k_le_kmax_half"] = {
        k: [round(float(v), 4) for v in (avg[k][ks] / avg["fp32_dm"][ks] - 1)] for k in ("fp32_learned", "fp32_none")}
    out["spectrum_max_rel_diff_all_shells"] = {
        k: float(np.abs(avg[k][1:kmax + 1] / avg["fp32_dm"][1:kmax + 1] - 1).max()) for k in ("fp32_learned",
                                                                                          "fp32_none")}
    out["network"] = src
    return out


def closure_training_rate(steps=300, batch=8192, n=1 << 21):
    """Adam training throughput of the closure network (samples/s) on
    synthetic features, with the backward contractions on the tensor cores
    and, for comparison, on the CUDA cores (host clock around
    sam_gpu_mlp_train, which synchronises)."""
    import numpy as np
    from sam_gb300 import SamGpu
    from sam_gb300 import closure_data as CD
    rng = np.random.default_rng(0)
    x = rng.standard_normal((n, 12)).astype(np.float32)
    y = (0.02 * np.abs(rng.standard_normal((n, 2)))).astype(np.float32)
    g = SamGpu(nx=16, ny=16, nz=16)
    out = {"batch": batch, "steps": steps, "unit": "samples/s"}
    try:
        for name, tc in (("tensor_cores", True), ("cuda_cores", False)):
            g.mlp_set(CD.init_params(0))
            g.mlp_set_backward(tc)
            g.mlp_train(x, y, 20, batch, 1e-3)  # warm-up
            t0 = time.perf_counter()
            g.mlp_train(x, y, steps, batch, 1e-3)
            out[name] = steps * batch / (time.perf_counter() - t0)
    finally:
        g.close()
    out["speedup"] = out["tensor_cores"] / out["cuda_cores"]
    return out


def ensemble_members(seed=5):
    """96 stratified-turbulence members of uneven sizes: 32 at 32^3, 32 at
    64^3, 24 at 96^3, 8 at 128^3; per member a seed, N uniform in [0.5, 4]
    (buoy_fac_z = N^2, lapse = 1), and the viscosity of a Taylor-microscale
    Reynolds number uniform in [50, 150] for the k^4 exp(-2 (k/4)^2) start
    field at rms velocity 1 (u' = 1, lambda = (5 E / Z)^(1/2) = 1/2, so
    nu = 0.5 / Re_lambda); FP32 bulk, CFL 0.5; the learned closure on the
    members of 96^3 and more."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for n, count in ((32, 32), (64, 32), (96, 24), (128, 8)):
        for _ in range(count):
            nn = rng.uniform(0.5, 4.0)
            re = rng.uniform(50.0, 150.0)
            out.append((dict(nx=n, ny=n, nz=n, i_strat=1, i_cfl=1, cfl0=0.5, vis=0.5 / re, pr=1.0, dt0=1e-3,
                             buoy_fac_z=nn * nn, lapse=1.0), int(rng.integers(1 << 30)), n >= 96))
    return out


def ensemble_form(K, W):
    """Aggregate member-steps/s of the 96-member ensemble: the 64 members
    without a closure in one persistent launch per RK3 stage and the 32
    learned-closure members in their own branches of the same step graph
    (tiles and FFT schedules from the ensemble autotuner, one tuning per
    member class); the same ensemble with every member in its own branch;
    the members run one after another in the same FP32 forms and tiles (the
    gain from running them together); and one after another in the plain
    FP64 drop-in."""
    import torch
    from sam_gb300 import SamEnsemble, SamGpu
    params, src = closure_params()
    members = ensemble_members()
    cfgs = [dict(cfg, precision=32) for cfg, _, _ in members]

    def timed_ensemble(persistent):
        ens = SamEnsemble(cfgs)
        try:
            ens.set_persistent(persistent)
            for m, (cfg, seed, learned) in enumerate(members):
                ens[m].init_random(seed, 6, 1.0, 6, 0.1)
                if learned:
                    ens[m].mlp_set(params)
                    ens[m].set_les(3)
            tuned = ens.autotune(3)  # setup, outside the timed region
            if persistent:
                class_tiles.update(tuned)
            ens.step(W)
            npers = ens.persistent_members()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ens.step(K)
            return time.perf_counter() - t0, npers
        finally:
            ens.close()

    class_tiles = {}
    t_ens, npers = timed_ensemble(True)
    t_br, _ = timed_ensemble(False)

    def sequential(cfg_of, closure):
        Ks = max(2, K // 4)
        total = 0.0
        for (cfg, seed, learned), c in zip(members, cfg_of):
            g = SamGpu(**c)
            g.init_random(seed, 6, 1.0, 6, 0.1)
            if closure and learned:
                g.mlp_set(params)
                g.set_les(3)
                t = dict(class_tiles.get((c["nx"], c["ny"], c["nz"], 32, 3), {}))
                if t:  # the ensemble's tiles for this class
                    sched = t.pop("fft_schedule")
                    g.set_tiles(**t)
                    g.set_fft_schedule(sched)
            g.step(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            g.step(Ks)
            torch.cuda.synchronize()
            total += (time.perf_counter() - t0) / Ks
            g.close()
        return len(members) / total

    seq32 = sequential(cfgs, True)
    seq64 = sequential([cfg for cfg, _, _ in members], False)
    agg = len(members) * K / t_ens
    return {"members": len(members), "sizes": {"32^3": 32, "64^3": 32, "96^3": 24, "128^3": 8},
            "value": agg, "unit": "member-steps/s", "precision": "FP32 bulk, learned closure on >= 96^3 (" + src + ")",
            "persistent_members": npers,
            "all_branches": {"value": len(members) * K / t_br, "unit": "member-steps/s",
                             "note": "every member its own branch of the step graph"},
            "sequential_fp32": {"value": seq32, "unit": "member-steps/s",
                                "note": "the same members and forms one after another"},
            "sequential_fp64_plain": {"value": seq64, "unit": "member-steps/s"}, "speedup": agg / seq64,
            "speedup_over_sequential_fp32": agg / seq32,
            "timing": "host clock around ensemble_step (it synchronises), after warm-up steps"}


def run_probe(args):
    """A short fixed launch sequence for ncu: init, 3 steps (each stage: the
    five passes), nothing else; --les 3 uses the LES start with the learned
    closure (network kernel launched at stage 1 of each step)."""
    from sam_gb300 import SamGpu, build as B
    B.build()
    if args.les:
        params, _ = closure_params()
        g = SamGpu(**les_cfg(args.precision))
        g.init_random(3, 6, 1.0, 6, 0.1)
        if args.les == 3:
            g.mlp_set(params)
        g.set_les(args.les)
    else:
        g = SamGpu(**workload_cfg(precision=args.precision))
        g.init_packet(PACKET["seed"], PACKET["k0"], PACKET["sigma"], PACKET["amplitude"], PACKET["noise"])
    g.step(3)
    print(json.dumps({"probe": True, "time": g.stats()["time"], "precision": args.precision, "les": args.les}))
    g.close()
    return 0


def run_parity_curve(args):
    """Error of the GPU forms (FP64, double-float, FP32 bulk) against the
    oracle versus step count on the 128^3 stratified decaying-turbulence
    configuration (N = 1, Pr = 1,
    nu = 1/800, k^4 exp(-2 (k/4)^2) start at rms 1 with theta at 0.1, CFL
    0.5), seeds 0, 1, 2: max over fields of max |u_gpu - u_oracle| / max
    |u_oracle| every `every` steps up to args.parity_curve steps; one JSON
    line.  Diagnostic mode (no timing)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from sam_gb300 import SamGpu, build as B
    B.build()
    O.build()
    cfg = dict(nx=128, ny=128, nz=128, i_strat=1, i_cfl=1, cfl0=0.5, vis=1.0 / 800, pr=1.0, buoy_fac_z=1.0,
               lapse=1.0)
    every = 25
    out = {"parity_curve": "128^3 stratified decaying turbulence, config of the 500-step run", "every": every,
           "measure": "max over fields of max|u_gpu - u_oracle| / max|u_oracle| (Nz_min rows)", "seeds": {}}
    for seed in (0, 1, 2):
        # the oracle's states every `every` steps, then each GPU form in turn
        # from the same start (one library context at a time)
        o = O.Oracle(**cfg)
        u = o.init_random(seed, 6, 1.0, 6, 0.1)
        u0 = u.copy(order="F")
        r = o.wave(o.d.lr)
        snaps, times = [], []
        done = 0
        while done < args.parity_curve:
            o.steps(u, r, every)
            done += every
            snaps.append(u.copy(order="F"))
            times.append(o.stats()["time"])
        nz_min, lu = o.d.nz_min, o.d.lu
        o.close()
        rows = [{"step": every * (i + 1), "time": times[i]} for i in range(len(snaps))]
        for prec in (64, 48, 32):
            g = SamGpu(precision=prec, **cfg)
            g.upload(u0)
            for i, ref in enumerate(snaps):
                g.step(every)
                ug = g.download()
                rows[i][f"prec{prec}"] = max(float(np.abs(ug[:nz_min, ..., n] - ref[:nz_min, ..., n]).max()
                                                  / np.abs(ref[:nz_min, ..., n]).max()) for n in range(lu))
            g.close()
        out["seeds"][str(seed)] = rows
    print(json.dumps(out), flush=True)
    return 0


def run_reference(args):
    rank, _, ws = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    steps = max(1, min(args.steps, 20))
    rate, secs, _, _, _ = cpu_oracle_rate(N, steps, threads, warm_stages=min(args.warmup, 3))
    sample = f"{steps} full RK3 steps of the 256^3 workload after {min(args.warmup, 3)} warm-up stage(s)"
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": "steps/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 / rate, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "grid": [N, N, N], "fields": 4},
            "cpu_baseline": {"value": rate, "unit": "steps/s", "cores": threads, "kind": "port",
                             "sample": sample + " (oracle: C restatement; the Fortran/MPI reference is "
                                                "unbuildable here: no Fortran compiler or MPI)"},
            "e2e": {"value": rate, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--no-dd", action="store_true", help="skip the double-float form")
    ap.add_argument("--no-les", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--grid", type=int, default=256, help="N of the N^3 box (profiling of smaller cases)")
    ap.add_argument("--precision", type=int, default=64, choices=[64, 48, 32],
                    help="precision of the timed run (32 for profiling the FP32 bulk form)")
    ap.add_argument("--probe", action="store_true",
                    help="profiling case: the workload's start state and 3 steps only (no timing, autotune or "
                         "baselines); with --les 3 the learned-closure LES start")
    ap.add_argument("--les", type=int, default=0, help="closure model of the --probe run")
    ap.add_argument("--parity-curve", type=int, default=0,
                    help="diagnostic: GPU-vs-oracle error every 25 steps up to this many steps at 128^3")
    args = ap.parse_args()
    global N, WORKLOAD
    if args.grid != N:
        WORKLOAD = WORKLOAD.replace("256^3", f"{args.grid}^3")
        N = args.grid
    if args.impl == "reference":
        return run_reference(args)
    if args.probe:
        return run_probe(args)
    if args.parity_curve:
        return run_parity_curve(args)

    rank, local_rank, ws = dist_env()
    if ws > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local_rank)
    import numpy as np
    import torch
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist

    from sam_gb300 import SamGpu
    from sam_gb300 import build as B
    B.build()

    K, W = args.steps, max(args.warmup, 3)
    stream = torch.cuda.Stream()
    g = SamGpu(**workload_cfg(precision=args.precision))
    g.set_stream(stream.cuda_stream)
    g.init_packet(PACKET["seed"], PACKET["k0"], PACKET["sigma"], PACKET["amplitude"], PACKET["noise"])
    u_init = g.download()
    tiles = g.autotune(3)  # setup, outside the timed region
    g.step(W)
    torch.cuda.synchronize()

    def barrier():
        if pg:
            pg.barrier()

    # ---- timed region: K steps from the resident state
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks() as clk:
        barrier()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            e0.record(stream)
            g.step(K)
            e1.record(stream)
        torch.cuda.synchronize()
        barrier()
    ms = max_over_ranks(e0.elapsed_time(e1), pg)
    value = whole_job_rate(K, ms / 1e3, ws)
    st = g.stats()
    launches_per_step = 3 * 5 + 1  # five passes per stage, vel_max completion at stage 1
    u_fp64 = g.download()

    # ---- per-pass durations (CUDA events between the passes of un-graphed stages)
    prof = [g.profile_stage(nrk, max(2, K // 4)) for nrk in (1, 2, 3)]
    passes = {k: sum(p[k] for p in prof) / 3 for k in prof[0]}
    fp64_peak = g.fp64_peak_tflops()

    # ---- e2e through the C ABI with pinned host buffers
    nbytes = u_init.nbytes
    pinned = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    uh = np.frombuffer(pinned.numpy(), dtype=np.complex128).reshape(u_init.shape, order="F")
    uh[...] = u_init
    g.set_stream(0)
    g.upload(uh)
    g.step(1)
    g.download()
    Ke = max(3, K // 2)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(Ke):
        g.upload(uh)
        g.step(1)
        g.download(out=uh)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, pg)
    mx, my, mz = dims()
    io_bytes = 4 * mx * my * mz * 16
    e2e = {"value": whole_job_rate(Ke, e2e_s, ws), "unit": "steps/s", "h2d_bytes_per_step": io_bytes,
           "d2h_bytes_per_step": io_bytes,
           "path": "sam_gpu_upload + sam_gpu_step(1) + sam_gpu_download on pinned host arrays"}
    g.close()

    # ---- FP32 bulk on the same workload and start state
    fp32 = None
    if not args.no_fp32:
        g32 = SamGpu(**workload_cfg(precision=32))
        g32.set_stream(stream.cuda_stream)
        g32.upload(u_init)
        tiles32 = g32.autotune(3)
        g32.step(W)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            e0.record(stream)
            g32.step(K)
            e1.record(stream)
        torch.cuda.synchronize()
        ms32 = e0.elapsed_time(e1)
        u32 = g32.download()
        prof32 = [g32.profile_stage(nrk, max(2, K // 4)) for nrk in (1, 2, 3)]
        passes32 = {k: sum(p[k] for p in prof32) / 3 for k in prof32[0]}
        err = [float(np.abs(u32[..., n] - u_fp64[..., n]).max() / np.abs(u_fp64[..., n]).max()) for n in range(4)]
        bands = band_errors(u32, u_fp64)
        g32.close()
        b32 = algorithmic_bytes_per_step(w=4)
        fp32 = {"value": ws * K / (ms32 / 1e3), "unit": "steps/s", "ms_per_step": ms32 / K,
                "rel_err_vs_fp64_per_field": err, "rel_l2_err_vs_fp64_per_field_and_band": bands,
                "after_steps": W + K,
                "hbm_gbs": b32 / (ms32 / K / 1e3) / 1e9, "passes_ms": passes32, "tiles": tiles32,
                # stages 2 and 3: the x pass alone (vel_max's kernels run at stage 1)
                "_x_ms": (prof32[1]["x_pass"] + prof32[2]["x_pass"]) / 2}

    # ---- the double-float form (FP32 pairs on the FP32 pipe, FP64-accurate)
    # on the same workload and start state
    ddf = None
    if not args.no_dd:
        gd = SamGpu(**workload_cfg(precision=48))
        gd.set_stream(stream.cuda_stream)
        gd.upload(u_init)
        tilesd = gd.autotune(3)
        gd.step(W)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            e0.record(stream)
            gd.step(K)
            e1.record(stream)
        torch.cuda.synchronize()
        msd = e0.elapsed_time(e1)
        ud = gd.download()
        profd = [gd.profile_stage(nrk, max(2, K // 4)) for nrk in (1, 2, 3)]
        passesd = {k: sum(p[k] for p in profd) / 3 for k in profd[0]}
        errd = [float(np.abs(ud[..., n] - u_fp64[..., n]).max() / np.abs(u_fp64[..., n]).max()) for n in range(4)]
        gd.close()
        bd = algorithmic_bytes_per_step(w=8)
        ddf = {"value": ws * K / (msd / 1e3), "unit": "steps/s", "ms_per_step": msd / K,
               "speedup_over_fp64": (ws * K / (msd / 1e3)) / value,
               "rel_err_vs_fp64_per_field": errd, "after_steps": W + K,
               "hbm_gbs": bd / (msd / K / 1e3) / 1e9, "passes_ms": passesd, "tiles": tilesd,
               "arithmetic": "FP32 pairs (hi + lo, about 48 significand bits) on the FP32 pipe; vel_max sums, "
                             "dt and the integrating factor's exponentials in FP64",
               "_x_ms": (profd[1]["x_pass"] + profd[2]["x_pass"]) / 2}

    # ---- the LES forms of the same workload: FP64 drop-in with dm.f's
    # dynamic Smagorinsky coupled in, and FP32 bulk with the learned closure
    les = None
    if not args.no_les:
        les = les_forms(stream, max(K, 20), W)
        les["closure_training"] = closure_training_rate()
    ens = None
    if not args.no_ensemble:
        ens = ensemble_form(max(4, K // 2), W)

    # ---- CPU baseline: the oracle on the host cores, bounded sample; its
    # final state is the parity reference of the same steps on the GPU
    cpu = None
    parity = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, secs, u_or, st_or, nz_min = cpu_oracle_rate(N, 2, threads, u_start=u_init)
        cpu = {"value": rate, "unit": "steps/s", "cores": threads, "kind": "port",
               "sample": f"2 full RK3 steps of the same 256^3 workload ({secs:.1f} s), oracle C restatement"}
        parity = parity_vs_oracle(u_init, u_or, st_or, nz_min, 2, stream)

    if rank != 0:
        return 0
    peaks = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    xb = x_pass_bytes()
    x_ms = passes["x_pass"]
    achieved = xb / (x_ms / 1e3) / 1e9
    tr = profile_traffic()
    alu = x_pass_flops() / (x_ms / 1e3) / 1e12
    roofline = {"bound": "fp64_alu", "kernel": "k_x_pass<double> (C2R, vel_max, 9 products, R2C)",
                "achieved": alu, "peak": fp64_peak, "unit": "TFLOP/s", "frac": alu / fp64_peak,
                "peak_source": "FP64 FMA peak measured live in this run (DFMA loop); not in MEASURED_PEAKS.json",
                "flops_per_launch": x_pass_flops(),
                "traffic": tr.get("bytes_per_launch") if tr else None,
                "hbm": {"achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                        "algorithmic_bytes_per_launch": xb,
                        "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if "hbm_gbs" in peaks
                        else "fallback"},
                "passes_ms": passes}
    if fp32 is not None:
        # the FP32 form's dominant kernel against the same HBM peak
        x32_ms = fp32.pop("_x_ms")
        xb32 = x_pass_bytes(w=4)
        a32 = xb32 / (x32_ms / 1e3) / 1e9
        tr32 = profile_traffic("x_pass_fp32_traffic.json")
        xk = "k_x_pass_f256" if N == 256 else "k_x_pass<float>"
        fp32["roofline"] = {"bound": "hbm", "kernel": xk + " (C2R, 9 products, R2C; stages 2 and 3)",
                            "achieved": a32, "peak": hbm_peak, "unit": "GB/s", "frac": a32 / hbm_peak,
                            "traffic": tr32.get("bytes_per_launch") if tr32 else None,
                            "algorithmic_bytes_per_launch": xb32, "ms": x32_ms,
                            "note": "bound by shared-memory traffic and latency: counters at 256^3 in "
                                    "profiles/x_pass_f256_fp32_256_ncu.md"}
    if ddf is not None:
        xd_ms = ddf.pop("_x_ms")
        ad = x_pass_bytes(w=8) / (xd_ms / 1e3) / 1e9
        ddf["roofline"] = {"bound": "fp32_issue", "kernel": "k_x_pass<dd> (C2R, 9 products, R2C; stages 2 and 3)",
                           "achieved_hbm_gbs": ad, "peak_hbm_gbs": hbm_peak, "hbm_frac": ad / hbm_peak,
                           "algorithmic_bytes_per_launch": x_pass_bytes(w=8), "ms": xd_ms,
                           "fp64_equivalent_tflops": x_pass_flops() / (xd_ms / 1e3) / 1e12,
                           "fp64_peak_tflops": fp64_peak}
    ms_step = ms / K
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": K, "warmup": W,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {64: "f64", 48: "f32 pairs (double-float)", 32: "f32"}[args.precision],
            "data": "synthetic (seeded, generated on the device)",
            "config": {"workload": WORKLOAD, "grid": [N, N, N], "fields": 4, "products": 9,
                       "l2": "inputs larger than L2 (state 161 MB, pencils up to 811 MB per pass)",
                       "parallelism": f"replicas x{ws}" if ws > 1 else "1 GPU",
                       "grid_point_updates_per_s": value * N ** 3,
                       "hbm_gbs_step": algorithmic_bytes_per_step() / (ms_step / 1e3) / 1e9,
                       "dt_final": st["dt"], "tiles": tiles},
            "roofline": roofline, "cpu_baseline": cpu, "parity_vs_oracle": parity, "e2e": e2e,
            "gpu_launches": launches_per_step * K,
            "clocks": clk.summary(), "double_float": ddf, "fp32_bulk": fp32, "les": les, "ensemble": ens}
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
