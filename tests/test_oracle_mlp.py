"""The warm-start network's CPU restatement (oracle/oracle.py) against
finite differences in float64: the backward formulas the tensor-core
training kernels implement."""
import numpy as np


def test_mlp_gradient_matches_finite_differences(orc):
    rng = np.random.default_rng(0)
    p = (rng.normal(size=orc.MLP_PARAMS) * 0.3).astype(np.float64)
    P = orc.mlp_unpack(p)
    P["W3"][3:] = 0
    P["b3"][3:] = 0
    p = orc.mlp_pack(P).astype(np.float64)
    X = rng.normal(size=(40, 16))
    X[:, 12:] = 0
    t = rng.normal(size=(40, 3))
    T = np.concatenate([t / np.linalg.norm(t, axis=1, keepdims=True), (rng.random((40, 1)) < 0.8)], axis=1)
    _, loss, g = orc.mlp_forward_backward(p, X, T, round_bf16=False)
    idx = rng.choice(np.flatnonzero(g != 0), 40, replace=False)
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        _, lp, _ = orc.mlp_forward_backward(q, X, T, round_bf16=False)
        q[i] -= 2 * h
        _, lm, _ = orc.mlp_forward_backward(q, X, T, round_bf16=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(g[i])) + 1e-7, (i, fd, g[i])


def test_bf16_rounding_is_nearest_even(orc):
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e-3], np.float32)
    y = orc.bf16(x)
    assert y[0] == 1.0 and y[1] == 1.0 and y[2] == 1.0 + 2 ** -7 and y[3] == -2.5
    assert abs(y[4] - 3.0e-3) < 3.0e-3 * 2 ** -8
