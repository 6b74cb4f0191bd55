"""Device kernels of the warm-start network against the CPU oracle (mlp_oracle)."""
import numpy as np
import pytest

import mlp_oracle as M

pytestmark = pytest.mark.gpu


def _data(n, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, M.NIN)).astype(np.float32)
    T = rng.standard_normal((n, M.NOUT)).astype(np.float32)
    return X, T


def test_forward_matches_oracle(eb):
    from endobeams_gb300 import warm_start as W
    p = M.init_params(0, out_gain=1.0)
    X, _ = _data(1000)
    Y = W.mlp_forward(p, X)
    R = M.forward(p, X)
    # FP32 accumulation over at most 128 terms against float64: relative 1e-4
    assert np.abs(Y - R).max() <= 1e-4 * max(1.0, np.abs(R).max())


def test_gradient_matches_oracle(eb):
    """Gradient check of the hand-written backward kernels against the CPU oracle
    (same bfloat16 weights; tolerance 2e-4 of the gradient's max norm)."""
    from endobeams_gb300 import warm_start as W
    p = M.init_params(1, out_gain=1.0)
    X, T = _data(777, 1)  # not a multiple of the 32-row tile
    T[5, :] = np.nan
    loss, g = W.mlp_loss_grad(p, X, T)
    rl, rg = M.loss_grad(p, X, T)
    assert abs(loss - rl) <= 1e-5 * rl
    for a, b in ((M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2), (M.OFF_B2, M.OFF_W3),
                 (M.OFF_W3, M.OFF_B3), (M.OFF_B3, M.NPARAMS)):
        ref = rg[a:b]
        assert np.abs(g[a:b] - ref).max() <= 2e-4 * np.abs(ref).max(), (a, b)


def test_training_reduces_loss_and_is_reproducible(eb):
    from endobeams_gb300 import warm_start as W
    rng = np.random.default_rng(7)
    X = rng.standard_normal((20000, M.NIN)).astype(np.float32)
    A = rng.standard_normal((M.NIN, M.NOUT)) / np.sqrt(M.NIN)
    T = (np.tanh(X @ A) + 0.1 * (X[:, :M.NOUT] ** 2)).astype(np.float32)
    p0 = M.init_params(2)
    p1, l1 = W.mlp_train(p0, X, T, epochs=6, batch=1024, lr=2e-3, seed=11)
    p2, l2 = W.mlp_train(p0, X, T, epochs=6, batch=1024, lr=2e-3, seed=11)
    assert np.array_equal(p1, p2) and np.array_equal(l1, l2)
    base = float(np.mean((M.forward(p0, X) - T) ** 2))
    after = float(np.mean((M.forward(p1, X) - T) ** 2))
    assert l1[-1] < l1[0] and after < 0.2 * base, (base, after, l1)
