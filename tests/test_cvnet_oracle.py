"""CPU tests of the control-variate network's oracle (oracle/cvnet_oracle.py):
its float64 backward pass against central finite differences, the bf16
rounding helper, and the loss minimisers."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import cvnet_oracle as N


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 1e-30, 3.0e38], np.float32)
    r = N.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0  # exactly halfway between 1 and 1 + 2^-7: ties to even
    assert r[2] == np.float32(1.0 + 2 ** -7)
    assert r[3] == -2.5
    u = N.bf16(np.random.default_rng(0).standard_normal(1000).astype(np.float32)).view(np.uint32)
    assert (u & 0xFFFF == 0).all()


def _problem(rows=24, G=3, seed=0):
    rng = np.random.default_rng(seed)
    p = N.init_params(seed).astype(np.float64)
    p[N.OFF_W4:N.OFF_B4] = rng.normal(0, 0.05, N.NOUT * N.HID)
    p[N.OFF_B1:N.OFF_W2] = rng.normal(0, 0.1, N.HID)
    f = rng.uniform(-1, 1, (rows, N.NFEAT))
    lab = np.zeros((rows, G, 8))
    A = rng.normal(size=(rows, G, 3, 3))
    C = np.einsum("rgij,rgkj->rgik", A, A)  # SPD covariance of (X, Ya, Yb)
    lab[..., 0], lab[..., 1], lab[..., 2] = C[..., 0, 0], C[..., 1, 1], C[..., 2, 2]
    lab[..., 3], lab[..., 4], lab[..., 5] = C[..., 0, 1], C[..., 0, 2], C[..., 1, 2]
    lab[..., 6] = rng.uniform(0.5, 2.0, (rows, G))
    lab[..., 7] = rng.uniform(0.5, 2.0, (rows, G))
    return p, f, lab


def test_fp64_backward_matches_finite_differences():
    p, f, lab = _problem()
    scales, ridge = (1.3, 0.9, 1.1), 0.05

    def loss(q):
        out, _ = N.forward(q, f, mimic=False)
        return sum(N.loss_grad(out, lab, scales, ridge)[0])

    g, _, _ = N.gradient(p, f, lab, scales, ridge, mimic=False)
    rng = np.random.default_rng(1)
    blocks = [(N.OFF_W1, N.NFEAT), (N.OFF_B1, N.HID), (N.OFF_W2, N.HID * N.HID), (N.OFF_B3, N.HID),
              (N.OFF_W4, N.NOUT * N.HID), (N.OFF_B4, N.NOUT)]
    h = 1e-6
    for off, n in blocks:
        for e in rng.choice(n, 6, replace=False):
            q = p.copy()
            q[off + e] += h
            lp = loss(q)
            q[off + e] -= 2 * h
            lm = loss(q)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[off + e]) <= 1e-6 + 1e-5 * abs(fd), (off, e, fd, g[off + e])


def test_padding_columns_get_zero_gradient():
    p, f, lab = _problem()
    g, _, _ = N.gradient(p, f, lab, (1, 1, 1), 0.0, mimic=True)
    W1 = g[N.OFF_W1:N.OFF_B1].reshape(N.HID, N.K0)
    assert np.all(W1[:, N.NFEAT:] == 0)


def test_loss_minimisers():
    """beta loss is minimised by the regression coefficients of X on (Ya, Yb);
    the log heads by o = log(E[label] / S)."""
    _, _, lab = _problem(rows=1, G=1, seed=3)
    y = lab[0, 0]
    C = np.array([[y[1], y[5]], [y[5], y[2]]])
    bstar = np.linalg.solve(C, [y[3], y[4]])
    out = np.zeros((1, N.NOUT))
    out[0, 0], out[0, 1] = bstar[0] - 1, bstar[1] + 1
    out[0, 2], out[0, 3] = np.log(y[6] / 0.7), np.log(y[7] / 1.9)
    _, d = N.loss_grad(out, lab[:, :1], (1.0, 0.7, 1.9), 0.0)
    np.testing.assert_allclose(d[0, :4], 0.0, atol=1e-9)
