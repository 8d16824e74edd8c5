"""The numpy restatement of the warm-start MLP (the gradient oracle) against finite differences."""
import numpy as np

from oracle import mlp_ref


def test_reference_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    n_params = sum(i * j + j for i, j in mlp_ref.DIMS)
    p = rng.normal(scale=0.1, size=n_params)
    x = rng.normal(size=(16, 48))
    t = rng.normal(size=(16, 3))
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    loss, g = mlp_ref.loss_and_grads(p, x, t, quantize=False)
    idx = rng.choice(n_params, 40, replace=False)
    for i in idx:
        e = np.zeros(n_params)
        e[i] = 1e-6
        lp, _ = mlp_ref.loss_and_grads(p + e, x, t, quantize=False)
        lm, _ = mlp_ref.loss_and_grads(p - e, x, t, quantize=False)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.01171875, -3.14159, 0.0], np.float32)
    r = mlp_ref.bf16(v)
    # 1 + 2^-8 and 1 + 3 * 2^-8 are halfway cases: ties go to the even mantissa
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.015625
    assert abs(r[3] + 3.140625) < 1e-9 and r[4] == 0.0
