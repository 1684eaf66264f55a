"""numpy restatement of the learned subgrid closure -- TEST INFRASTRUCTURE ONLY.

The closure network is new (the reference has no learned model; its sm.f /
dm.f are the eddy-viscosity models the network stands beside).  This module
restates, in float64 numpy with the same BF16 roundings, what the CUDA
library computes, so the tests can check the tensor-core forward pass, the
backward pass and the coupled step:

  x  = bf16(features)                      12 inputs
  h1 = bf16(relu(x W1^T + b1))             64
  h2 = bf16(relu(h1 W2^T + b2))            64
  o  = h2 W3^T + b3                        2
  C  = 0.02 softplus(o)                    (C_nu, C_kappa)

with W1, W2, W3 rounded to BF16 and the biases in FP32.  The loss is
L = (1/(2n)) sum over points and outputs of (C - y)^2.  The features are the
invariants of the strain S, vorticity w and buoyancy gradient g defined in
`features` below (the same formulas as the CUDA feature pass).
"""
from __future__ import annotations

import numpy as np

N_IN, N_H, N_OUT = 12, 64, 2
SCALE = 0.02
OFF_W1 = 0
OFF_B1 = OFF_W1 + N_H * N_IN
OFF_W2 = OFF_B1 + N_H
OFF_B2 = OFF_W2 + N_H * N_H
OFF_W3 = OFF_B2 + N_H
OFF_B3 = OFF_W3 + N_OUT * N_H
N_PARAMS = OFF_B3 + N_OUT


def bf16(x) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(p):
    p = np.asarray(p)
    if p.dtype != np.float64:
        p = p.astype(np.float32)
    return (p[OFF_W1:OFF_B1].reshape(N_H, N_IN), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(N_H, N_H),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3].reshape(N_OUT, N_H), p[OFF_B3:N_PARAMS])


def init_params(seed=0):
    """He-style initial weights, zero biases; the last layer starts small."""
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, dtype=np.float32)
    p[OFF_W1:OFF_B1] = rng.standard_normal(N_H * N_IN) * np.sqrt(2.0 / N_IN)
    p[OFF_W2:OFF_B2] = rng.standard_normal(N_H * N_H) * np.sqrt(2.0 / N_H)
    p[OFF_W3:OFF_B3] = rng.standard_normal(N_OUT * N_H) * 0.1 * np.sqrt(1.0 / N_H)
    return p


def softplus(x):
    return np.where(x > 20, x, np.log1p(np.exp(np.minimum(x, 20))))


def forward(p, feats, rnd=True):
    """rnd=False drops the BF16 roundings (exact float64 network, for the
    finite-difference check of `grad`)."""
    q = bf16 if rnd else (lambda a: np.asarray(a, dtype=np.float64))
    w1, b1, w2, b2, w3, b3 = unpack(p)
    x = q(feats).astype(np.float64)
    h1 = q(np.maximum(x @ q(w1).T.astype(np.float64) + b1, 0)).astype(np.float64)
    h2 = q(np.maximum(h1 @ q(w2).T.astype(np.float64) + b2, 0)).astype(np.float64)
    o = h2 @ q(w3).T.astype(np.float64) + b3
    return SCALE * softplus(o), h1, h2, o


def grad(p, feats, target, rnd=True):
    """Gradient of L with respect to the FP32 parameter vector (through the
    BF16 weights as straight-through roundings) and L itself."""
    q = bf16 if rnd else (lambda a: np.asarray(a, dtype=np.float64))
    w1, b1, w2, b2, w3, b3 = unpack(p)
    n = len(feats)
    c, h1, h2, o = forward(p, feats, rnd)
    x = q(feats).astype(np.float64)
    r = c - target
    loss = 0.5 * (r ** 2).sum() / n
    sig = 1.0 / (1.0 + np.exp(-o))
    dout = r / n * SCALE * sig
    d2 = (dout @ q(w3).astype(np.float64)) * (h2 > 0)
    d1 = (d2 @ q(w2).astype(np.float64)) * (h1 > 0)
    g = np.zeros(N_PARAMS)
    g[OFF_W1:OFF_B1] = (d1.T @ x).ravel()
    g[OFF_B1:OFF_W2] = d1.sum(0)
    g[OFF_W2:OFF_B2] = (d2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = d2.sum(0)
    g[OFF_W3:OFF_B3] = (dout.T @ h2).ravel()
    g[OFF_B3:N_PARAMS] = dout.sum(0)
    return g, loss
