"""The FP64 denoiser oracle's backward pass against finite differences (CPU)."""
import numpy as np

from oracle import unet_oracle as U


def _setup(seed=0, n=1, h=8, w=8):
    rng = np.random.default_rng(seed)
    p = U.init_params(seed).astype(np.float64)
    # non-zero biases and a live output layer so every path carries gradient
    for (wt, b), (ci, co, _) in zip(U.split_params(p), U.LAYERS):
        b[:] = rng.uniform(-0.05, 0.2, co)
    x = rng.uniform(-1, 1, (n, h, w, 16))
    t = rng.uniform(0, 3, (n, h, w, 4))
    return p, x, t


def test_param_count_matches_layer_table():
    assert U.param_count() == sum(9 * ci * co + co for ci, co, _ in U.LAYERS)
    assert U.init_params(0).size == U.param_count()


def test_backward_matches_finite_differences():
    p, x, t = _setup()
    _, cache = U.forward(p, x)
    loss, g = U.backward(cache, t)
    assert np.isclose(loss, U.loss_only(p, x, t))
    rng = np.random.default_rng(1)
    offs = np.cumsum([0] + [9 * ci * co + co for ci, co, _ in U.LAYERS])
    idx = []
    for li in range(len(U.LAYERS)):
        ci, co, _ = U.LAYERS[li]
        lo = offs[li]
        # two weights and one bias per layer (output layer: live channels only)
        k = rng.integers(0, 9 * ci)
        c = rng.integers(0, 3 if li == len(U.LAYERS) - 1 else co)
        idx += [lo + k * co + c, lo + rng.integers(0, 9 * ci) * co + c, lo + 9 * ci * co + c]
    eps = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += eps
        lp = U.loss_only(q, x, t)
        q[i] -= 2 * eps
        lm = U.loss_only(q, x, t)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_dgrad_is_adjoint_of_conv():
    rng = np.random.default_rng(2)
    x = rng.standard_normal((2, 5, 7, 16))
    w = rng.standard_normal((9, 16, 32))
    g = rng.standard_normal((2, 5, 7, 32))
    lhs = np.sum(U.conv3x3(x, w) * g)
    assert np.isclose(lhs, np.sum(x * U.conv3x3_dgrad(g, w)))
    assert np.isclose(lhs, np.sum(w * U.conv3x3_wgrad(x, g)))


def test_bf16_rounding_ties_to_even():
    vals = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.0e38], np.float32)
    got = U.bf16(vals)
    assert got[0] == 1.0 and got[1] == 1.0          # tie -> even (down)
    assert got[2] == np.float32(1.0 + 4 * 2 ** -8)  # tie -> even (up)
    assert got[3] == -2.5
