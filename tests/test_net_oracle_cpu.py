"""The proposal network's CPU restatement: its analytic gradient agrees with finite
differences of its own loss (without BF16 rounding), which pins the restatement the
GPU kernels are compared with."""
from __future__ import annotations

import numpy as np

from oracle import net_oracle


def _loss(p, x, t):
    out, _ = net_oracle.forward(p, x, rounding=False)
    _, (lf, lc, _) = net_oracle.loss_grad(out, t, rounding=False)
    return lf + 0.25 * lc


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    n = sum(co * 9 * ci + co for ci, co in zip(net_oracle.CIN, net_oracle.COUT))
    p = rng.normal(0, 0.15, n).astype(np.float64).astype(np.float32)
    shape = (1, 11, 12)  # wider than the largest dilation (8), so every tap reaches in
    x = rng.uniform(-1, 1, shape + (net_oracle.CIN[0],)).astype(np.float32)
    t = np.zeros(shape + (3,), np.float32)
    t[..., 0] = rng.normal(0, 3, shape)
    t[..., 1] = rng.normal(0, 3, shape)
    t[..., 2] = 1.0
    out, acts = net_oracle.forward(p, x, rounding=False)
    dY, _ = net_oracle.loss_grad(out, t, rounding=False)
    g = net_oracle.backward(p, x, acts, dY, rounding=False)
    idx = rng.choice(n, 40, replace=False)
    eps = 1e-3
    num = []
    for i in idx:
        q = p.astype(np.float64).copy()
        q[i] += eps
        lp = _loss(q.astype(np.float32), x, t)
        q[i] -= 2 * eps
        lm = _loss(q.astype(np.float32), x, t)
        num.append((lp - lm) / (2 * eps))
    num = np.array(num)
    # the confidence label is held fixed by the analytic gradient; compare the bulk
    rel = np.linalg.norm(num - g[idx]) / np.linalg.norm(num)
    assert rel < 5e-2, rel


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.01171875, -2.5, 3.14159], np.float32)
    assert list(net_oracle.bf16(v)) == [1.0, 1.0, 1.015625, -2.5, 3.140625]
