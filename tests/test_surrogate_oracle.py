"""The CPU restatement of the surrogate (oracle/surrogate_ref.py) checked against itself:
the FP64 backward against finite differences, the BF16 rounding, and the invariances the
features are built to have."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import surrogate_ref as S  # noqa: E402


def random_theta(rng, scale=0.3):
    th = rng.normal(scale=scale, size=S.N_PARAMS)
    th[S.OFF_W1 + 13 * S.N_HID:S.OFF_W2] = 0.0
    return th


def random_inputs(rng, n):
    X = np.zeros((n, 16))
    X[:, :12] = rng.uniform(-1, 1, size=(n, 12))
    X[:, 12] = 1.0
    return X


def test_fp64_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    th = random_theta(rng)
    X = random_inputs(rng, 40)
    t = rng.normal(size=40)
    g, loss = S.backward(th, X, t, emulate=False)
    idx = np.concatenate([rng.choice(np.arange(S.OFF_W1, S.OFF_W1 + 13 * 64), 12, replace=False),
                          rng.choice(np.arange(S.OFF_W2, S.N_PARAMS), 40, replace=False), [S.OFF_B4]])
    h = 1e-6
    for k in idx:
        tp, tm = th.copy(), th.copy()
        tp[k] += h
        tm[k] -= h
        lp = S.backward(tp, X, t, emulate=False)[1]
        lm = S.backward(tm, X, t, emulate=False)[1]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])


def test_bf16_rounding_ties_to_even():
    one = np.float32(1.0)
    ulp = np.float32(2.0 ** -7)                  # BF16 spacing at 1
    vals = np.array([1.0, 1 + 2.0 ** -8, 1 + 3 * 2.0 ** -8, 1 + 2.0 ** -7 + 2.0 ** -8, -2.5, 3.0e-20], np.float32)
    out = S.bf16(vals)
    assert out[0] == one
    assert out[1] == one                          # tie -> even
    assert out[2] == one + 2 * ulp                # above the tie
    assert out[3] == one + 2 * ulp                # tie -> even (odd mantissa rounds up)
    assert out[4] == np.float32(-2.5)
    assert abs(out[5] - vals[5]) <= abs(vals[5]) * 2.0 ** -8


def _rand_unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _perp(rng, a):
    v = _rand_unit(rng, len(a))
    v -= (v * a).sum(1, keepdims=True) * a
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _rot(rng):
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    return q * np.sign(np.linalg.det(q))


def test_features_invariant_under_rotation_and_axis_flip():
    rng = np.random.default_rng(3)
    n = 400
    a1, a2 = _rand_unit(rng, n), _rand_unit(rng, n)
    p1, p2 = _perp(rng, a1), _perp(rng, a2)
    r = rng.uniform(-2.5, 2.5, size=(n, 3))
    h = np.full(n, 1.5, np.float32)
    tc = np.zeros(n, np.float32)
    f0, d0 = S.pair_features(r, a1, p1, h, tc, a2, p2, h, tc)
    R = _rot(rng)
    f1, _ = S.pair_features(r @ R.T, a1 @ R.T, p1 @ R.T, h, tc, a2 @ R.T, p2 @ R.T, h, tc)
    # the direction between nearly touching segments is ill-conditioned in FP32
    ok = f0[:, 0] > 0.05
    assert ok.sum() > 300
    assert np.allclose(f0[ok], f1[ok], atol=2e-5)
    # flipping an axis leaves a spherocylinder (and the patch wedge around it) unchanged
    f2, _ = S.pair_features(r, -a1, p1, h, tc, -a2, p2, h, tc)
    keep = (np.abs(f0[:, 2]) > 1e-3) & (np.abs(f0[:, 3]) > 1e-3) & ok
    assert np.allclose(f0[keep], f2[keep], atol=2e-5)


def test_segment_distance_feature_matches_fp64():
    rng = np.random.default_rng(5)
    n = 300
    a1, a2 = _rand_unit(rng, n), _rand_unit(rng, n)
    r = rng.uniform(-3, 3, size=(n, 3))
    h = np.full(n, 1.5, np.float32)
    f, d2 = S.pair_features(r, a1, _perp(rng, a1), h, np.zeros(n, np.float32), a2, _perp(rng, a2), h,
                            np.zeros(n, np.float32))
    # brute-force FP64 closest distance on a fine grid of the two segments
    s = np.linspace(-1.5, 1.5, 301)
    for k in range(0, n, 30):
        P = r[k][None, None, :] + s[:, None, None] * a1[k] - s[None, :, None] * a2[k]
        dmin = np.sqrt((P ** 2).sum(-1).min())
        assert f[k, 0] <= dmin + 1e-4 and f[k, 0] >= dmin - 0.02
