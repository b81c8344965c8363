"""The denoiser's tensor-core kernels against the FP64 oracle (GPU).

Inputs and weights are rounded to bfloat16 exactly as the library rounds
them, so single layers differ from the oracle only by FP32 accumulation and
the final BF16 store (2^-9 relative).  The whole network additionally rounds
every stored activation to BF16; its gradients are compared per layer by
relative L2 error.
"""
import numpy as np
import pytest

from oracle import unet_oracle as U
from pt_gb300 import abi
from pt_gb300.denoise import UNet, init_params

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(params=["rows", "tap"], autouse=True)
def conv_kernel(request, monkeypatch):
    """Every test runs on both convolution kernels: the persistent halo-reuse
    kernel (default) and the one-tile-per-CTA kernel (PT_CONV_KERNEL=tap)."""
    if request.param == "tap":
        monkeypatch.setenv("PT_CONV_KERNEL", "tap")
    else:
        monkeypatch.delenv("PT_CONV_KERNEL", raising=False)
    return request.param


def dev(a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to("cuda").to(dtype).contiguous()


def host(t):
    return t.float().cpu().numpy().astype(np.float64)


def lib():
    return abi.lib()


def check(rc):
    assert rc == 0, lib().pt_unet_last_error(None).decode()


CONV_SHAPES = [  # n, h, w, pitch, c0, cin, cout
    (1, 8, 8, 16, 0, 16, 32),
    (2, 20, 40, 48, 16, 32, 16),
    (1, 16, 136, 224, 0, 224, 96),
    (1, 12, 24, 96, 0, 96, 224),
    (3, 4, 4, 64, 32, 32, 128),
    (2, 8, 12, 64, 0, 64, 64),
    (1, 10, 20, 160, 0, 160, 64),
    (2, 16, 24, 96, 0, 96, 32),
]


@pytest.mark.parametrize("shape", CONV_SHAPES)
def test_conv_forward_matches_oracle(shape):
    n, h, w, pitch, c0, cin, cout = shape
    rng = np.random.default_rng(cin * 7 + cout)
    x = U.bf16(rng.uniform(-1, 1, (n, h, w, pitch)))
    wt = (rng.standard_normal((9, cin, cout)) * np.sqrt(2.0 / (9 * cin))).astype(np.float32)
    b = rng.uniform(-0.1, 0.1, cout).astype(np.float32)
    xd, wd, bd = dev(x, torch.bfloat16), dev(wt, torch.float32), dev(b, torch.float32)
    out = torch.full((n, h, w, cout), 7.0, dtype=torch.bfloat16, device="cuda")
    for relu in (0, 1):
        check(lib().pt_nn_conv3x3(xd.data_ptr(), n, h, w, pitch, c0, cin, wd.data_ptr(), bd.data_ptr(), cout, relu,
                                  out.data_ptr(), None))
        ref = U.conv3x3(x[..., c0:c0 + cin].astype(np.float64), U.bf16(wt).astype(np.float64), b)
        if relu:
            ref = np.maximum(ref, 0.0)
        got = host(out)
        tol = 2.0 ** -8 * np.abs(ref) + 1e-4 * np.sqrt(np.mean(ref ** 2))
        bad = np.abs(got - ref) > tol
        assert not bad.any(), f"{bad.sum()} of {bad.size} outside tolerance; max err {np.abs(got - ref).max():.3g}"


@pytest.mark.parametrize("shape", CONV_SHAPES)
def test_conv_dgrad_matches_oracle(shape):
    n, h, w, _, _, cin, cout = shape
    if cout > 128 or cin > 256:
        pytest.skip("layer shape not used backward")
    rng = np.random.default_rng(cin + 3 * cout)
    g = U.bf16(rng.standard_normal((n, h, w, cout)))
    wt = (rng.standard_normal((9, cin, cout)) * np.sqrt(2.0 / (9 * cin))).astype(np.float32)
    mask = U.bf16(rng.uniform(-1, 1, (n, h, w, cin)))
    gd, wd, md = dev(g, torch.bfloat16), dev(wt, torch.float32), dev(mask, torch.bfloat16)
    out = torch.full((n, h, w, cin), 7.0, dtype=torch.bfloat16, device="cuda")
    for use_mask in (False, True):
        check(lib().pt_nn_conv3x3_dgrad(gd.data_ptr(), n, h, w, cout, wd.data_ptr(), cin,
                                        md.data_ptr() if use_mask else None, out.data_ptr(), None))
        ref = U.conv3x3_dgrad(g.astype(np.float64), U.bf16(wt).astype(np.float64))
        if use_mask:
            ref = ref * (mask > 0)
        got = host(out)
        tol = 2.0 ** -8 * np.abs(ref) + 1e-4 * np.sqrt(np.mean(ref ** 2))
        bad = np.abs(got - ref) > tol
        assert not bad.any(), f"{bad.sum()} of {bad.size} outside tolerance; max err {np.abs(got - ref).max():.3g}"


WGRAD_SHAPES = [  # n, h, w, pitch, c0, cin, cout
    (2, 16, 24, 16, 0, 16, 32),
    (1, 8, 136, 224, 0, 224, 96),
    (1, 4, 4, 48, 16, 32, 16),
    (4, 32, 32, 160, 0, 160, 64),
]


@pytest.mark.parametrize("shape", WGRAD_SHAPES)
def test_conv_wgrad_matches_oracle(shape):
    n, h, w, pitch, c0, cin, cout = shape
    rng = np.random.default_rng(pitch + cout)
    x = U.bf16(rng.uniform(-1, 1, (n, h, w, pitch)))
    g = U.bf16(rng.standard_normal((n, h, w, cout)))
    xd, gd = dev(x, torch.bfloat16), dev(g, torch.bfloat16)
    dw = torch.zeros((9, cin, cout), dtype=torch.float32, device="cuda")
    check(lib().pt_nn_conv3x3_wgrad(xd.data_ptr(), n, h, w, pitch, c0, cin, gd.data_ptr(), cout, dw.data_ptr(), None))
    ref = U.conv3x3_wgrad(x[..., c0:c0 + cin].astype(np.float64), g.astype(np.float64))
    got = dw.cpu().numpy().astype(np.float64)
    tol = 1e-5 * np.abs(ref) + 1e-5 * np.abs(ref).max()
    bad = np.abs(got - ref) > tol
    assert not bad.any(), f"{bad.sum()} of {bad.size} outside tolerance; max err {np.abs(got - ref).max():.3g}"


def _net_inputs(seed, n, h, w):
    rng = np.random.default_rng(seed)
    p = init_params(seed)
    offs = np.cumsum([0] + [9 * ci * co + co for ci, co, _ in U.LAYERS])
    for li, (ci, co, _) in enumerate(U.LAYERS):
        p[offs[li] + 9 * ci * co: offs[li + 1]] = rng.uniform(-0.05, 0.2, co)
    x = U.bf16(rng.uniform(-1, 1, (n, h, w, 16)))
    t = rng.uniform(0, 3, (n, h, w, 4)).astype(np.float32)
    return p, x, t


def _weights_bf16(p):
    q = p.astype(np.float64).copy()
    for w, _ in U.split_params(q):
        w[...] = U.bf16(w)
    return q


def test_unet_gradients_match_oracle():
    """Forward, loss and every layer's gradient of the whole network.

    Single layers round like the exact result to within 1-3 BF16 ulp on
    <0.2 % of outputs (the element-wise tests above).  Through the network
    those rare flips, and the ReLU masks they flip, compound chaotically in
    the backward pass: the two convolution kernels, both exact per layer,
    differ from each other by up to ~4 % at the first layers.  Against an
    oracle that rounds to BF16 wherever the library stores BF16: 6 % per
    layer; against the exact FP64 network, where BF16 storage alone moves
    the middle layers by ~10 %: 20 %.  Wiring errors (a wrong channel offset,
    a missing mask) show up as O(1) errors."""
    n, h, w = 2, 16, 24
    p, x, t = _net_inputs(3, n, h, w)
    net = UNet(n, h, w)
    net.set_params(p)
    net.input_tensor().copy_(dev(x, torch.bfloat16))
    base = np.random.default_rng(4).uniform(0, 1.5, (n, h, w, 4)).astype(np.float32)
    base[..., 3] = 0
    net.base_tensor().copy_(dev(base, torch.float32))
    tgt = dev(t, torch.float32)
    net.forward()
    loss = net.backward(tgt.data_ptr())
    g = net.grads().astype(np.float64)
    got_out = net.output_tensor().cpu().numpy().astype(np.float64)
    pw = _weights_bf16(p)
    offs = np.cumsum([0] + [9 * ci * co + co for ci, co, _ in U.LAYERS])
    report = []
    for storage, tol_out, tol_loss, tol_g in ((True, 0.005, 0.002, 0.06), (False, 0.03, 0.02, 0.20)):
        ref_out, cache = U.forward(pw, x.astype(np.float64), bf16_storage=storage, base=base.astype(np.float64))
        ref_loss, ref_g = U.backward(cache, t)
        assert np.abs(got_out - ref_out).max() <= tol_out * np.abs(ref_out).max() + 1e-4
        assert abs(loss - ref_loss) <= tol_loss * ref_loss
        rels = []
        for li in range(len(U.LAYERS)):
            a, b = g[offs[li]:offs[li + 1]], ref_g[offs[li]:offs[li + 1]]
            rels.append(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))
        report.append(rels)
        assert max(rels) < tol_g, f"bf16_storage={storage}: per-layer relative gradient error {np.round(rels, 4)}"
    print("per-layer relative gradient error (bf16-storage oracle, fp64 oracle):", np.round(report, 4))


def test_training_reduces_loss():
    """A few hundred Adam steps fit a smooth synthetic mapping."""
    n, h, w = 4, 32, 32
    rng = np.random.default_rng(5)
    x = rng.uniform(0, 1, (n, h, w, 16)).astype(np.float32)
    x[..., 11:] = 0
    # target: linear radiance whose log is a fixed mix of the input channels
    mix = rng.uniform(-0.5, 0.5, (16, 3))
    t = np.expm1(np.clip(x @ mix + 0.5, 0, 3)).astype(np.float32)
    t = np.concatenate([t, np.ones((n, h, w, 1), np.float32)], axis=-1)
    net = UNet(n, h, w)
    net.set_params(init_params(1))
    net.input_tensor().copy_(dev(U.bf16(x), torch.bfloat16))
    tgt = dev(t, torch.float32)
    losses = []
    for step in range(300):
        net.forward()
        losses.append(net.backward(tgt.data_ptr()))
        net.adam(1e-3)
    assert np.isfinite(losses).all()
    assert np.mean(losses[-10:]) < 0.2 * np.mean(losses[:3]), (losses[:3], losses[-10:])
