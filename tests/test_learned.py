"""Learned preconditioner network: the CPU oracle (finite differences, BF16 rounding)."""
import numpy as np

from oracle.mlp import bf16, forward, loss_and_gradients


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    W = [rng.standard_normal((16, 12)), rng.standard_normal((12, 12)), rng.standard_normal((12, 16))]
    X = rng.standard_normal((7, 16))
    T = rng.standard_normal((7, 16))
    _, g = loss_and_gradients(W, X, T, round_bf16=False)
    for layer in range(3):
        for (i, j) in [(0, 0), (3, 5), (11, 7)]:
            Wp = [w.copy() for w in W]
            Wm = [w.copy() for w in W]
            Wp[layer][i, j] += 1e-6
            Wm[layer][i, j] -= 1e-6
            fd = (loss_and_gradients(Wp, X, T, False)[0] - loss_and_gradients(Wm, X, T, False)[0]) / 2e-6
            assert abs(fd - g[layer][i, j]) < 1e-5 * max(1.0, abs(fd)), (layer, i, j)


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -9, -2.5, 1e-40, np.inf], dtype=np.float32)
    r = bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2.0 ** -7 and r[3] == -2.5 and r[5] == np.inf
    y = np.random.default_rng(1).standard_normal(1000).astype(np.float32)
    rel = np.abs(bf16(y) - y) / np.abs(y)
    assert rel.max() <= 2.0 ** -8 + 1e-12


def test_forward_is_positively_homogeneous():
    # bias-free ReLU network: MLP(a x) = a MLP(x) for a > 0 (the preconditioner relies on it
    # to be independent of the scale of the Krylov vector)
    rng = np.random.default_rng(2)
    W = [rng.standard_normal((8, 6)), rng.standard_normal((6, 6)), rng.standard_normal((6, 8))]
    X = rng.standard_normal((4, 8))
    assert np.allclose(forward(W, 3.5 * X, False)[2], 3.5 * forward(W, X, False)[2])
