"""The learned load balancer's FP64 restatement, pinned on the CPU: its
gradient against central finite differences, and its bf16 rounding."""
import numpy as np

import instances
import lbm_oracle as lo


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.0, 0.0, 1e-3], dtype=np.float64)
    got = lo.bf16(x)
    # 1 + 2^-8 is halfway between 1 and 1 + 2^-7: ties to even -> 1.0
    assert got[0] == 1.0 and got[1] == 1.0
    # 1 + 1.5 * 2^-8 rounds up to 1 + 2^-7
    assert got[2] == 1.0078125
    assert got[3] == -3.0 and got[4] == 0.0
    assert abs(got[5] - 1e-3) / 1e-3 < 2 ** -8


def test_features_are_one_hot_cells():
    w = 4
    goal = np.arange(16, dtype=np.uint8)[None]
    f = lo.features(goal, w)
    assert f.tolist() == [[(t - 1) * 16 + t for t in range(1, 16)]]


def _params(width, seed):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.05, lo.num_params(width))
    W1, b1, W2, b2, w3, b3 = lo.split(p, width)
    b1 += 0.05
    b2 += 0.05
    return p


def test_fp64_gradient_matches_finite_differences():
    w = 4
    tiles = instances.random_walks(w, 12, 20, seed=5)
    slack = np.arange(12) % 5
    target = np.linspace(1.0, 9.0, 12)
    p = _params(w, 1)
    loss, _, g = lo.forward_backward(p, tiles, slack, target, w, rounding=False)
    assert loss > 0
    rng = np.random.default_rng(2)
    d = lo.feature_dim(w)
    # coordinates in every parameter group; W1 rows that the batch touches
    f = lo.features(tiles, w)
    touched = np.unique(np.concatenate([f.reshape(-1), [d - 1]]))
    offs = np.cumsum([0, d * 256, 256, 256 * 256, 256, 256, 1])
    coords = list(rng.choice(touched, 8) * 256 + rng.integers(0, 256, 8))
    for grp in range(1, 6):
        coords += list(rng.integers(offs[grp], offs[grp + 1], 6))
    eps = 1e-6
    for c in coords:
        q = p.copy()
        q[c] += eps
        lp = lo.forward_backward(q, tiles, slack, target, w, rounding=False)[0]
        q[c] -= 2 * eps
        lm = lo.forward_backward(q, tiles, slack, target, w, rounding=False)[0]
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[c]) <= 1e-6 + 1e-4 * abs(fd), (c, fd, g[c])


def test_rounded_gradient_close_to_exact():
    w = 5
    tiles = instances.random_walks(w, 16, 30, seed=6)
    slack = np.arange(16) % 4
    target = np.linspace(2.0, 12.0, 16)
    p = _params(w, 3)
    _, _, g0 = lo.forward_backward(p, tiles, slack, target, w, rounding=False)
    _, _, g1 = lo.forward_backward(p, tiles, slack, target, w, rounding=True)
    assert np.linalg.norm(g1 - g0) <= 0.05 * np.linalg.norm(g0)
