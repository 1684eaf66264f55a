"""Generate tests/golden/kats.json from the reference's own known-answer tests.

Run where the reference tree is available, naming its root directory:
    python tests/golden/make_golden.py <reference-root>

The reference ships no data files beyond input.dat, so the fixtures are:
  * tfftpk: FFTPACK's self test (fft.f:2838-3011): rfftf of N=36 ones is
    (36, 0, ..., 0); rfftb of a unit impulse is all ones; tolerance as there.
  * tst_transpose: spectral -> physical -> spectral identity per mode with the
    tolerance 1e-15 of tst_transpose.f:124.
  * gw_input_dat: the reference's input.dat case (a single plane internal
    gravity wave, i_prob = -4).  The wave parameters follow init.f:184-210; a
    lone plane wave has no nonlinear self-interaction, so with vis = 0 every
    stored coefficient evolves by the RK3 amplification factor
    G = 1 + z + z^2/2 + z^3/6, z = i omega_i dt, per step (gw.tex:139-150
    gives omega_i^2 = N^2 sin^2 beta).
  * initial divergence bound 1e-7 (initial_field.f:147).
"""
import json
import math
import os
import sys


def read_input_dat(path):
    vals = {}
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 2 and not parts[0].startswith("#"):
                vals[parts[0].lower()] = parts[1]
    return vals


def main(ref_root):
    v = read_input_dat(os.path.join(ref_root, "input.dat"))
    nx, ny, nz = int(v["nx"]), int(v["ny"]), int(v["nz"])
    xl, yl, zl = float(v["xl"]), float(v["yl"]), float(v["zl"])
    grav, lapse0, to = float(v["grav"]), float(v["lapse0"]), float(v["to"])
    gam, lambda_x = float(v["gam"]), float(v["lambda_x"])
    dt0, n_steps = float(v["dt0"]), int(v["n_steps"])
    amplitude, uo, vis = float(v["amplitude"]), float(v["uo"]), float(v["vis"])
    # init.f:184-228 (i_gw_type = 0: Gam and lambda_x given)
    two_pi = 2.0 * math.pi
    k_w = -two_pi / lambda_x
    m_w = -gam * abs(k_w)
    n_sq = grav * lapse0 / to
    omega_i = math.sqrt(n_sq / (1.0 + gam ** 2))
    lambda_z = two_pi / abs(m_w)
    xl = round(xl / lambda_x) * lambda_x
    zl = round(zl / lambda_z) * lambda_z
    z = complex(0.0, omega_i * dt0)
    g = 1 + z + z * z / 2 + z ** 3 / 6
    gn = g ** n_steps
    out = {
        "source": "generated by tests/golden/make_golden.py from the reference's input.dat and fft.f",
        "tfftpk": {"n": 36, "tol": 0.01},
        "tst_transpose": {"tol": 1.0e-15},
        "initial_divergence_max": 1.0e-7,
        "gw_input_dat": {
            "nx": nx, "ny": ny, "nz": nz, "xl": xl, "yl": yl, "zl": zl,
            "grav": grav, "lapse0": lapse0, "to": to, "gam": gam, "lambda_x": lambda_x,
            "lambda_z": lambda_z, "k_w": k_w, "m_w": m_w, "omega_i": omega_i,
            "amplitude": amplitude, "uo": uo, "vis": vis, "dt": dt0, "n_steps": n_steps,
            "n_dealias": int(v["n_dealias"]), "nrk_max": int(v["nrk_max"]), "i_strat": int(v["i_strat"]),
            "rk3_amplification_re": gn.real, "rk3_amplification_im": gn.imag,
        },
    }
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kats.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference-root>")
    main(sys.argv[1])
