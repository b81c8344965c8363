"""FP64 restatement of the denoiser network — TEST INFRASTRUCTURE ONLY.

The reference (anveba/pt) has no denoiser, so there is no reference file to
follow: this module restates, in float64 numpy, the network that
include/pt_denoise.h documents (layer table, parameter layout, pooling,
upsampling, concatenation order and loss), so that tests can check the
library's BF16 tensor-core forward and backward passes against it.  Only
tests/ import it.  Its own backward pass is checked against central finite
differences in tests/test_unet_oracle.py.

Layout: activations NHWC float64; weights w[9][c_in][c_out] with tap =
3*ky + kx, bias b[c_out]; parameters of all layers concatenated in layer
order, each as w then b.
"""
from __future__ import annotations

import numpy as np

# (c_in, c_out, relu), layer order of pt_unet_layer_shape
LAYERS = [(16, 32, True), (32, 32, True), (32, 64, True), (64, 64, True), (64, 96, True), (96, 96, True),
          (96, 128, True), (128, 128, True), (224, 96, True), (96, 96, True), (160, 64, True), (64, 64, True),
          (96, 32, True), (32, 32, True), (32, 16, False)]
LOSS_CLAMP = 16.0


def param_count() -> int:
    return sum(9 * ci * co + co for ci, co, _ in LAYERS)


def split_params(p: np.ndarray):
    """Views (w [9, ci, co], b [co]) per layer."""
    out, off = [], 0
    for ci, co, _ in LAYERS:
        w = p[off:off + 9 * ci * co].reshape(9, ci, co)
        off += 9 * ci * co
        b = p[off:off + co]
        off += co
        out.append((w, b))
    return out


def init_params(seed: int = 0) -> np.ndarray:
    """He-normal weights (fan-in 9 * c_in), zero biases; the output layer is
    scaled by 0.02 (the network starts close to the identity on its
    residual base) and its unused channels 3..15 are zero."""
    rng = np.random.default_rng(seed)
    parts = []
    for li, (ci, co, _) in enumerate(LAYERS):
        w = rng.standard_normal((9, ci, co)) * np.sqrt(2.0 / (9 * ci))
        if li == len(LAYERS) - 1:
            w *= 0.02
            w[:, :, 3:] = 0.0
        parts += [w.ravel(), np.zeros(co)]
    return np.concatenate(parts).astype(np.float32)


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float32."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


# ---------------------------------------------------------------- layers
def conv3x3(x: np.ndarray, w: np.ndarray, b: np.ndarray | None = None) -> np.ndarray:
    n, h, wd, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((n, h, wd, w.shape[2]))
    for tap in range(9):
        ky, kx = divmod(tap, 3)
        out += xp[:, ky:ky + h, kx:kx + wd, :] @ w[tap]
    if b is not None:
        out += b
    return out


def conv3x3_dgrad(g: np.ndarray, w: np.ndarray) -> np.ndarray:
    n, h, wd, _ = g.shape
    gp = np.pad(g, ((0, 0), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((n, h, wd, w.shape[1]))
    for tap in range(9):
        ky, kx = divmod(tap, 3)
        # x[p + off] contributed to out[p]; so dx[q] += g[q - off] w^T
        out += gp[:, 2 - ky:2 - ky + h, 2 - kx:2 - kx + wd, :] @ w[tap].T
    return out


def conv3x3_wgrad(x: np.ndarray, g: np.ndarray) -> np.ndarray:
    n, h, wd, ci = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    dw = np.zeros((9, ci, g.shape[3]))
    for tap in range(9):
        ky, kx = divmod(tap, 3)
        xs = xp[:, ky:ky + h, kx:kx + wd, :].reshape(-1, ci)
        dw[tap] = xs.T @ g.reshape(-1, g.shape[3])
    return dw


def _pool2(x):
    n, h, w, c = x.shape
    return x.reshape(n, h // 2, 2, w // 2, 2, c).mean(axis=(2, 4))


def pool2_backward(g):
    return np.repeat(np.repeat(g, 2, axis=1), 2, axis=2) * 0.25


def up2(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up2_backward(g):
    n, h, w, c = g.shape
    return g.reshape(n, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4))


# ---------------------------------------------------------------- network
def _keep(a):
    return a


def _store_bf16(a):
    return bf16(a).astype(np.float64)


def forward(params: np.ndarray, x: np.ndarray, bf16_storage: bool = False, base: np.ndarray | None = None):
    """Returns (out [n, h, w, 16], cache).  `base` ([n, h, w, 4], the residual
    base of pt_unet_base) is added to output channels 0-3.  With bf16_storage every tensor the
    library stores as BF16 (layer outputs, pooled maps, gradients) is rounded
    to BF16 where the library rounds it; the output layer stays FP32."""
    q = _store_bf16 if bf16_storage else _keep
    P = [(w.astype(np.float64), b.astype(np.float64)) for w, b in split_params(params)]
    c = {"x0": x.astype(np.float64), "q": q}

    def layer(i, inp):
        pre = conv3x3(inp, *P[i])
        if i == len(LAYERS) - 1:
            return pre
        return q(np.maximum(pre, 0.0) if LAYERS[i][2] else pre)

    def pool2(a):
        return q(_pool2(a))

    c["e0a"] = layer(0, c["x0"])
    c["e0b"] = layer(1, c["e0a"])
    c["p1"] = pool2(c["e0b"])
    c["e1a"] = layer(2, c["p1"])
    c["e1b"] = layer(3, c["e1a"])
    c["p2"] = pool2(c["e1b"])
    c["e2a"] = layer(4, c["p2"])
    c["e2b"] = layer(5, c["e2a"])
    c["p3"] = pool2(c["e2b"])
    c["b3a"] = layer(6, c["p3"])
    c["b3b"] = layer(7, c["b3a"])
    c["cat2"] = np.concatenate([up2(c["b3b"]), c["e2b"]], axis=3)
    c["d2a"] = layer(8, c["cat2"])
    c["d2b"] = layer(9, c["d2a"])
    c["cat1"] = np.concatenate([up2(c["d2b"]), c["e1b"]], axis=3)
    c["d1a"] = layer(10, c["cat1"])
    c["d1b"] = layer(11, c["d1a"])
    c["cat0"] = np.concatenate([up2(c["d1b"]), c["e0b"]], axis=3)
    c["d0a"] = layer(12, c["cat0"])
    c["d0b"] = layer(13, c["d0a"])
    c["out"] = layer(14, c["d0b"])
    if base is not None:
        c["out"][..., :4] += base
    c["P"] = P
    return c["out"], c


def loss_and_grad_out(out: np.ndarray, target: np.ndarray):
    """Loss of include/pt_denoise.h and its gradient w.r.t. the output."""
    t = np.maximum(target[..., :3].astype(np.float64), 0.0)
    y = np.log1p(t)
    wgt = (1.0 + np.minimum(t, LOSS_CLAMP)) ** 2
    d = out[..., :3] - y
    m = d.size
    loss = float(np.sum(wgt * d * d) / m)
    g = np.zeros_like(out)
    g[..., :3] = 2.0 * wgt * d / m
    return loss, g


def backward(cache, target: np.ndarray):
    """Returns (loss, flat fp64 gradient in parameter order)."""
    c, P, q = cache, cache["P"], cache["q"]
    loss, g_out = loss_and_grad_out(c["out"], target)
    g_out = q(g_out)
    grads = [None] * len(LAYERS)

    def lay(i, inp, g_pre):
        grads[i] = (conv3x3_wgrad(inp, g_pre), g_pre.sum(axis=(0, 1, 2)))
        return conv3x3_dgrad(g_pre, P[i][0])

    def relu_mask(g, z):
        return q(g * (z > 0))

    g = lay(14, c["d0b"], g_out)
    g = lay(13, c["d0a"], relu_mask(g, c["d0b"]))
    g_cat0 = q(lay(12, c["cat0"], relu_mask(g, c["d0a"])))
    g = relu_mask(up2_backward(g_cat0[..., :64]), c["d1b"])
    g = lay(11, c["d1a"], g)
    g_cat1 = q(lay(10, c["cat1"], relu_mask(g, c["d1a"])))
    g = relu_mask(up2_backward(g_cat1[..., :96]), c["d2b"])
    g = lay(9, c["d2a"], g)
    g_cat2 = q(lay(8, c["cat2"], relu_mask(g, c["d2a"])))
    g = relu_mask(up2_backward(g_cat2[..., :128]), c["b3b"])
    g = lay(7, c["b3a"], g)
    g_p3 = q(lay(6, c["p3"], relu_mask(g, c["b3a"])))
    g = relu_mask(g_cat2[..., 128:] + pool2_backward(g_p3), c["e2b"])
    g = lay(5, c["e2a"], g)
    g_p2 = q(lay(4, c["p2"], relu_mask(g, c["e2a"])))
    g = relu_mask(g_cat1[..., 96:] + pool2_backward(g_p2), c["e1b"])
    g = lay(3, c["e1a"], g)
    g_p1 = q(lay(2, c["p1"], relu_mask(g, c["e1a"])))
    g = relu_mask(g_cat0[..., 64:] + pool2_backward(g_p1), c["e0b"])
    g = lay(1, c["e0a"], g)
    lay(0, c["x0"], relu_mask(g, c["e0a"]))
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return loss, flat


def loss_only(params: np.ndarray, x: np.ndarray, target: np.ndarray) -> float:
    out, _ = forward(params, x)
    return loss_and_grad_out(out, target)[0]
