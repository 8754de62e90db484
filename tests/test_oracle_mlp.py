"""The MLP oracle's backward pass equals finite differences of its forward
pass (FP64), so it can serve as the checker of the GPU gradients."""

import numpy as np

from oracle import mlp


def _tiny_weights(rng, sizes=(5, 7, 6, 4, 2)):
    return [(rng.normal(0, 0.5, (a, b)), rng.normal(0, 0.1, b)) for a, b in zip(sizes, sizes[1:])]


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    weights = _tiny_weights(rng)
    x = rng.normal(size=(9, 5))
    t = rng.normal(size=(9, 2))

    def loss(ws):
        y, _ = mlp.forward(x, ws)
        return np.sum((y - t) ** 2) / x.shape[0]

    y, acts = mlp.forward(x, weights)
    grads, value = mlp.backward(acts, y, t, weights)
    assert np.isclose(value, loss(weights))
    eps = 1e-6
    for layer in range(4):
        for which in (0, 1):
            arr = weights[layer][which]
            flat = arr.reshape(-1)
            for idx in rng.choice(flat.size, size=min(5, flat.size), replace=False):
                old = flat[idx]
                flat[idx] = old + eps
                up = loss(weights)
                flat[idx] = old - eps
                down = loss(weights)
                flat[idx] = old
                fd = (up - down) / (2 * eps)
                got = grads[layer][which].reshape(-1)[idx]
                assert abs(fd - got) <= 1e-6 * max(1.0, abs(fd)), (layer, which, fd, got)


def test_bf16_rounding_is_nearest_even():
    vals = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 2.5e-30, 65504.0])
    out = mlp.bf16(vals)
    # bf16 keeps 8 significant bits: relative error below 2^-8
    assert np.all(np.abs(out - vals) <= np.abs(vals) * 2.0**-8 + 1e-45)
    assert mlp.bf16(1.0 + 2.0**-8) == 1.0          # tie rounds to even
    assert mlp.bf16(1.0 + 3 * 2.0**-8) == 1.0 + 2.0**-6
