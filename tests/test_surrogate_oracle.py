"""The surrogate's FP64 network restatement (oracle/mlp.py) against finite differences: pins the
checker that the GPU gradient tests use. CPU only."""
import numpy as np

from oracle import mlp


def _net(rng, dims):
    return [(rng.normal(0, 1 / np.sqrt(dims[l]), (dims[l + 1], dims[l])), rng.normal(0, 0.1, dims[l + 1]))
            for l in range(len(dims) - 1)]


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(5)
    dims = [6, 16, 16, 5]
    layers = _net(rng, dims)
    X = rng.normal(size=(32, 6))
    T = rng.normal(size=(32, 5))
    n_valid = 4
    loss, grads, _ = mlp.loss_and_grads(layers, X, T, n_valid)
    h = 1e-6
    for l, (W, b) in enumerate(layers):
        for arr, g in ((W, grads[l][0]), (b, grads[l][1])):
            flat, gflat = arr.reshape(-1), g.reshape(-1)
            for i in rng.choice(flat.size, size=min(6, flat.size), replace=False):
                old = flat[i]
                flat[i] = old + h
                lp = mlp.loss_and_grads(layers, X, T, n_valid)[0]
                flat[i] = old - h
                lm = mlp.loss_and_grads(layers, X, T, n_valid)[0]
                flat[i] = old
                fd = (lp - lm) / (2 * h)
                assert abs(fd - gflat[i]) <= 1e-6 * max(1.0, abs(fd)), (l, i, fd, gflat[i])


def test_forward_agrees_with_loss_pass_and_bf16_rounding():
    rng = np.random.default_rng(6)
    layers = _net(rng, [8, 12, 3])
    X = rng.normal(size=(10, 8))
    _, _, Y = mlp.loss_and_grads(layers, X, np.zeros((10, 3)), 3)
    assert np.array_equal(Y, mlp.forward(layers, X))
    x = np.array([1.0, 1.00390625, 1.001953125, 1.005859375, -3.0e-3, 0.0])
    # BF16 keeps 7 fraction bits: 1 + 2^-8 is a tie between 1 and 1 + 2^-7 (rounds to even: 1),
    # 1 + 2^-9 rounds down, 1 + 3 * 2^-9 is past the midpoint and rounds up
    assert list(mlp.bf16(x)[:4]) == [1.0, 1.0, 1.0, 1.0078125]
    assert mlp.bf16(x)[5] == 0.0
