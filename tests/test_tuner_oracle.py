"""The CPU restatement of the autotuner's features and cost-model gradient, pinned without a GPU:
features on hand-checked matrices, the gradient against central finite differences."""
import numpy as np

from oracle import tuner_oracle as TO


def test_features_hand_checked():
    # rows of lengths 0, 0, 0, 4 in a 4 x 8 matrix: Gini 0.75, mean 1, one empty-row fraction
    pos = np.array([0, 0, 0, 0, 4])
    crd = np.array([0, 3, 5, 7])
    f = TO.features(pos, crd, 8)
    assert f[0] == np.log2(5) and f[1] == np.log2(5) and f[2] == 1.0
    assert np.isclose(f[3], np.sqrt(3.0))            # std of (0,0,0,4) is sqrt(3), mean 1
    assert f[4] == np.log2(5) and np.isclose(f[5], 0.75)
    assert np.isclose(f[6], 4 / 8)                     # max |j - 3| = 4 (j = 7)
    assert np.isclose(f[7], (3 + 0 + 2 + 4) / 4 / 8)
    assert f[8] == 0.75 and f[9] == np.log2(9)


def test_features_equal_rows_and_empty():
    pos = np.arange(0, 101, 5)
    crd = np.tile(np.arange(5), 20)
    f = TO.features(pos, crd, 50)
    assert f[3] == 0.0 and abs(f[5]) < 1e-15 and f[8] == 0.0
    e = TO.features(np.zeros(1, np.int64), np.zeros(0, np.int64), 3)
    assert list(e[1:9]) == [0.0] * 8


def test_gini_log_bins_close_to_exact():
    rng = np.random.default_rng(5)
    L = np.concatenate([rng.integers(0, 50, 3000), rng.integers(3000, 200000, 40)])
    pos = np.concatenate([[0], np.cumsum(L)])
    crd = np.zeros(pos[-1], np.int64)
    g = TO.features(pos, crd, 1)[5]
    x = np.sort(L).astype(np.float64)
    n = len(x)
    exact = ((2 * np.arange(1, n + 1) - n - 1) * x).sum() / (n * x.sum())
    assert abs(g - exact) < 2e-3


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(7)
    n = 37
    X = rng.normal(size=(n, TO.F))
    Y = rng.normal(size=(n, TO.K))
    M = (rng.random((n, TO.K)) > 0.2).astype(np.float64)
    params = rng.normal(0, 0.3, TO.NPARAM)
    norm = np.concatenate([rng.normal(size=TO.F) * 0.1, 1 + rng.random(TO.F)])
    g = TO.grad(params, norm, X, Y, M)
    idx = rng.choice(TO.NPARAM, 120, replace=False)
    fd = TO.finite_difference(params, norm, X, Y, M, idx)
    assert np.max(np.abs(g[idx] - fd)) <= 1e-6 * max(1.0, np.max(np.abs(fd)))
