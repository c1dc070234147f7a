"""The MLP oracle's own gradient (FP64, no rounding) against central finite differences, and its
BF16 rounding helper against the bit-level definition."""

import numpy as np

import mlp_oracle as M


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = M.init_params(3).astype(np.float64)
    X = rng.normal(size=(64, 8))
    T = rng.normal(size=64) * 0.3
    _, g, _ = M.forward_backward(p, X, T, round_bf16=False)
    eps = 1e-6
    idx = rng.choice(M.NPARAMS, 60, replace=False)
    idx = np.concatenate([idx, [M.OB1, M.OB2, M.OB3, M.OW3]])
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += eps
        pm[k] -= eps
        fd = (M.forward_backward(pp, X, T, False)[0] - M.forward_backward(pm, X, T, False)[0]) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])) + 1e-8, (k, fd, g[k])


def test_bf16_rounding_is_nearest_even():
    vals = np.array([1.0, 1.00390625, 1.001953125, 1.005859375, -3.1415927, 65504.0], np.float32)
    r = M.bf16r(vals)
    # representable values stay, halfway cases go to even, others to nearest
    assert r[0] == 1.0 and r[1] == 1.0078125 or r[1] == 1.0
    assert r[2] == 1.0
    assert r[3] == 1.0078125
    assert abs(r[4] - (-3.140625)) < 1e-9
    u = np.asarray(r, np.float32).view(np.uint32)
    assert np.all((u & 0xFFFF) == 0)
