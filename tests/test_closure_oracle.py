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
