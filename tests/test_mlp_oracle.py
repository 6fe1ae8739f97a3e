"""The warm-start network's CPU oracle checked on its own (no GPU): bf16
rounding, analytic gradients against float64 finite differences, and the
first Adam step."""
import numpy as np

import mlp_oracle as mo


def test_bf16_rounding_ties_to_even():
    e = 2.0 ** -8
    x = np.array([1.0, 1 + e, 1 + 3 * e, -(1 + 3 * e), 3.0e38, 1e-40, 0.1])
    r = mo.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                    # halfway, mantissa stays even
    assert r[2] == 1 + 4 * e              # halfway, rounds up to the even neighbour
    assert r[3] == -(1 + 4 * e)
    assert np.isfinite(r[4])
    assert r[6] == np.float32(0.10009765625)


def _net(rng, dims):
    return [(rng.normal(0, 1 / np.sqrt(i), (o, i)), rng.normal(0, 0.1, o)) for i, o in zip(dims[:-1], dims[1:])]


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    params = _net(rng, [13, 16, 16, 16, 7])
    X = rng.normal(size=(9, 13))
    Y = rng.normal(size=(9, 7))
    assert mo.fd_check(params, X, Y, n_probe=40) < 1e-5


def test_gradients_with_linear_skip_match_finite_differences():
    rng = np.random.default_rng(7)
    params = _net(rng, [11, 16, 16, 5]) + [(rng.normal(0, 0.3, (5, 11)), None)]
    X = rng.normal(size=(8, 11))
    Y = rng.normal(size=(8, 5))
    assert mo.fd_check(params, X, Y, n_probe=40) < 1e-5
    y, _ = mo.forward(params, X, emulate=False)
    y0, _ = mo.forward(params[:-1], X, emulate=False)
    np.testing.assert_allclose(y - y0, X @ params[-1][0].T, atol=1e-12)


def test_metric_loss_gradients_match_finite_differences():
    rng = np.random.default_rng(8)
    params = _net(rng, [9, 16, 6]) + [(rng.normal(0, 0.3, (6, 9)), None)]
    A = rng.normal(size=(6, 4))
    X = rng.normal(size=(8, 9))
    Y = rng.normal(size=(8, 6))
    metric = (A, 0.01)
    _, g = mo.loss_and_grads(params, X, Y, emulate=False, metric=metric)
    h = 1e-5
    W = params[0][0]
    for idx in ((0, 0), (3, 5), (15, 8)):
        old = W[idx]
        W[idx] = old + h
        lp, _ = mo.loss_and_grads(params, X, Y, emulate=False, metric=metric)
        W[idx] = old - h
        lm, _ = mo.loss_and_grads(params, X, Y, emulate=False, metric=metric)
        W[idx] = old
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[0][0][idx]) <= 1e-6 * max(1.0, abs(fd))
    # the identity metric with lam 0 is the mean squared error
    l1, _ = mo.loss_and_grads(params, X, Y, emulate=False, metric=(np.eye(6), 0.0))
    l2, _ = mo.loss_and_grads(params, X, Y, emulate=False)
    assert abs(l1 - l2) <= 1e-12 * l2


def test_emulated_gradients_close_to_exact():
    rng = np.random.default_rng(4)
    params = _net(rng, [40, 32, 32, 24])
    X = rng.normal(size=(16, 40))
    Y = rng.normal(size=(16, 24))
    _, ge = mo.loss_and_grads(params, X, Y, emulate=True)
    _, gx = mo.loss_and_grads(params, X, Y, emulate=False)
    for (a, _), (b, _) in zip(ge, gx):
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 3e-2


def test_first_adam_step_moves_by_lr_times_sign():
    rng = np.random.default_rng(5)
    params = _net(rng, [6, 8, 3])
    X = rng.normal(size=(8, 6))
    Y = rng.normal(size=(8, 3))
    _, g = mo.loss_and_grads(params, X, Y, emulate=False)
    state = [tuple(np.zeros_like(p) for p in (W, W, b, b)) for W, b in params]
    new, _ = mo.adam_step(params, g, state, t=1, lr=1e-3)
    for (W0, b0), (W1, b1), (gW, gb) in zip(params, new, g):
        big = np.abs(gW) > 1e-6
        np.testing.assert_allclose((W0 - W1)[big], 1e-3 * np.sign(gW[big]), rtol=1e-3)
        np.testing.assert_allclose(b0 - b1, 1e-3 * np.sign(gb), rtol=1e-3)


def test_training_loop_of_the_oracle_reduces_loss():
    rng = np.random.default_rng(6)
    params = _net(rng, [5, 16, 16, 2])
    X = rng.normal(size=(64, 5))
    Y = np.stack([np.sin(X[:, 0]) + X[:, 1] * X[:, 2], X[:, 3] - 0.5 * X[:, 4]], axis=1)
    state = [tuple(np.zeros_like(p) for p in (W, W, b, b)) for W, b in params]
    l0, _ = mo.loss_and_grads(params, X, Y, emulate=False)
    for t in range(1, 301):
        _, g = mo.loss_and_grads(params, X, Y, emulate=False)
        params, state = mo.adam_step(params, g, state, t, lr=1e-2)
    l1, _ = mo.loss_and_grads(params, X, Y, emulate=False)
    assert l1 < 0.1 * l0
