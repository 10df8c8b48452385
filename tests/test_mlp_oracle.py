"""CPU checks of the network oracle (oracle/mlp.py) used to verify the device training kernels."""
import numpy as np

from oracle import mlp


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159265, 1e-3], dtype=np.float32)
    r = mlp.bf16_round(x)
    # every result is representable in BF16 (low 16 bits zero) and within half an ulp (2^-8 relative)
    assert not (r.view(np.uint32) & 0xFFFF).any()
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0 ** -8)
    assert r[1] == np.float32(1.0)  # tie 1 + 2^-8 rounds to even


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    dims = mlp.layer_dims(5, 7, 2, 3)
    n = sum(a * b + b for a, b in zip(dims[:-1], dims[1:]))
    p = rng.standard_normal(n).astype(np.float32) * 0.5
    # exactly BF16-representable weights make the straight-through gradient the true gradient
    p = mlp.bf16_round(p)
    x = rng.standard_normal((4, 5))
    t = rng.standard_normal((4, 3))
    loss, g = mlp.loss_grad(p, dims, x, t)
    # finite differences on the biases (not rounded) and on weights (rounding-free perturbation via biases)
    layers = np.cumsum([0] + [a * b + b for a, b in zip(dims[:-1], dims[1:])])
    for li, (a, b) in enumerate(zip(dims[:-1], dims[1:])):
        for j in range(b):
            k = layers[li] + a * b + j
            h = 1e-3
            pp = p.astype(np.float64).copy()
            pm = pp.copy()
            pp[k] += h
            pm[k] -= h
            fd = (mlp.loss_grad(pp.astype(np.float32), dims, x, t)[0] -
                  mlp.loss_grad(pm.astype(np.float32), dims, x, t)[0]) / (2 * h)
            assert abs(fd - g[k]) <= 1e-4 * max(1.0, abs(g[k]))
