"""The denoised pipeline on the GPU: what the trained network gains over plain
accumulation, and the input side's state rules.

The gain is measured on scenes the network never saw (the benchmark's mid
scene and the small scene, at 256x256) against 2048-spp references
accumulated in FP64 on the GPU, with the reference's meansq (RGB, n - 1).
"""
import numpy as np
import pytest

import pt_gb300 as P
from pt_gb300 import abi, scenes
from pt_gb300.denoise import WEIGHTS_DIR, UNet, init_params, load_params

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

W = H = 256
WEIGHTS = WEIGHTS_DIR / "unet.bin"


def meansq(img, ref):
    d = img[..., :3].astype(np.float64) - ref[..., :3]
    return float(np.sum(d * d) / (d.size - 1))


@pytest.fixture(scope="module")
def ctx():
    c = P.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def trained():
    if not WEIGHTS.exists():
        pytest.fail(f"trained weights missing: {WEIGHTS} (python -m pt_gb300.train_denoiser)")
    u = UNet(1, H, W)
    u.set_params(load_params(WEIGHTS))
    yield u
    u.close()


@pytest.mark.parametrize("which", ["mid", "small"])
def test_trained_network_beats_plain_accumulation(ctx, trained, which, tmp_path):
    make = scenes.mid_scene if which == "mid" else scenes.small_scene
    hs = P.HostScene.load(make(tmp_path / which, seed=1 if which == "mid" else 0))
    ctx.upload(hs.pack())
    ctx.build_accel()
    ctx.render(hs.render_params(W, H, 2048, 8, accum_mode=abi.PT_ACCUM_FP32_FP64), stats=False)
    ref = ctx.read_image(fp64=True)
    gains = {}
    for spp in (2, 4, 8):
        p = hs.render_params(W, H, spp, 8)
        ctx.render_denoised(trained, p)
        den = ctx.read_denoised()
        plain = ctx.read_image()  # the same samples, undenoised
        gains[spp] = (meansq(plain, ref), meansq(den, ref))
        assert np.isfinite(den).all()
    for spp, (m_plain, m_den) in gains.items():
        assert m_den < m_plain / 3.0, f"{which} at {spp} spp: plain {m_plain:.3g}, denoised {m_den:.3g}"
    print(which, {k: (round(a, 5), round(b, 5), round(a / b, 1)) for k, (a, b) in gains.items()})


def test_untrained_network_does_not_help(ctx, tmp_path):
    """The gain comes from training: the freshly initialised network (output
    layer near zero, so close to the identity on its residual base) leaves
    the noisy image's error where it was."""
    hs = P.HostScene.load(scenes.small_scene(tmp_path / "s", seed=0))
    ctx.upload(hs.pack())
    ctx.build_accel()
    ctx.render(hs.render_params(W, H, 1024, 8, accum_mode=abi.PT_ACCUM_FP32_FP64), stats=False)
    ref = ctx.read_image(fp64=True)
    u = UNet(1, H, W)
    u.set_params(init_params(0))
    ctx.render_denoised(u, hs.render_params(W, H, 4, 8))
    m_den, m_plain = meansq(ctx.read_denoised(), ref), meansq(ctx.read_image(), ref)
    u.close()
    assert m_den > 0.5 * m_plain


def test_input_packing_and_snapshot_rules(ctx):
    raw, cam = scenes.tiny_raw("two_tris")
    hs = P.HostScene.from_raw(raw, cam)
    fresh = P.Context(0)
    buf = torch.zeros((32, 40, 16), dtype=torch.bfloat16, device="cuda")
    base = torch.zeros((32, 40, 4), dtype=torch.float32, device="cuda")
    fresh.upload(hs.pack())
    fresh.build_accel()
    p = hs.render_params(40, 32, 4, 4)
    fresh.render(p)
    with pytest.raises(P.PtError) as e:  # no features yet
        fresh.denoise_input(4, buf.data_ptr())
    assert e.value.status == abi.PT_ERR_STATE
    fresh.render_features(p)
    fresh.denoise_input(4, buf.data_ptr(), base.data_ptr())
    x = buf.float().cpu().numpy()
    img = fresh.read_image()
    assert np.allclose(base.cpu().numpy()[..., :3], np.log1p(np.maximum(img[..., :3], 0)), rtol=1e-6, atol=1e-7)
    assert np.all(x[..., 14] == 0) and np.all(x[..., 11:14] == 0)  # no snapshot: no noise estimate
    assert np.allclose(x[..., 10], np.log2(4) / 8, atol=1e-2)
    # a snapshot of the first half, then the second half continues the image
    fresh.render(hs.render_params(40, 32, 2, 4))
    fresh.denoise_snapshot()
    fresh.render(hs.render_params(40, 32, 2, 4, sample_index=2))
    fresh.denoise_input(4, buf.data_ptr())
    x = buf.float().cpu().numpy()
    assert np.all(x[..., 14] == 1) and np.abs(x[..., 11:14]).max() > 0
    two_calls = buf.clone()
    # the armed snapshot, taken inside one 4-sample render, gives the same input bit for bit
    assert abi.lib().pt_denoise_snapshot_at(fresh._h, 2) == abi.PT_OK
    fresh.render(hs.render_params(40, 32, 4, 4))
    fresh.denoise_input(4, buf.data_ptr())
    assert torch.equal(buf.view(torch.int16), two_calls.view(torch.int16))
    # a fresh image invalidates the snapshot
    fresh.render(hs.render_params(40, 32, 4, 4))
    fresh.denoise_input(4, buf.data_ptr())
    assert np.all(buf.float().cpu().numpy()[..., 14] == 0)
    # the network must match the image size
    u = UNet(1, 64, 64)
    with pytest.raises(P.PtError) as e:
        fresh.denoise(u, 4)
    assert e.value.status == abi.PT_ERR_INVALID
    u.close()
    fresh.close()


def test_features_accumulated_in_render(ctx, tmp_path):
    """PT_RENDER_FEATURES: the same feature means from the wavefront and the
    megakernel, the image unchanged by the flag, and the features close to the
    stand-alone pass over the same camera rays."""
    hs = P.HostScene.load(scenes.small_scene(tmp_path / "f", seed=0))
    ctx.upload(hs.pack())
    ctx.build_accel()
    out = {}
    for name, kern in (("wave", abi.PT_KERNEL_WAVEFRONT), ("mega", abi.PT_KERNEL_MEGA)):
        p = hs.render_params(64, 48, 5, 6, kernel=kern)
        ctx.render(p)
        plain = ctx.read_image().copy()
        p.flags = abi.PT_RENDER_FEATURES
        ctx.render(p)
        assert np.array_equal(plain.view(np.uint32), ctx.read_image().view(np.uint32))
        out[name] = ctx.read_features()
    for a, b in zip(out["wave"], out["mega"]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    ctx.render_features(hs.render_params(64, 48, 5, 6))
    sa, sn = ctx.read_features()
    fa, fn = out["wave"]
    assert np.allclose(fa, sa, rtol=1e-5, atol=1e-6) and np.allclose(fn, sn, rtol=1e-5, atol=1e-6)
    assert fa[..., 3].max() > 0 and np.abs(fn[..., :3]).max() > 0.5


def test_fp16_feature_storage(ctx, trained, tmp_path):
    """PT_RENDER_FEATURES_FP16: features and the armed snapshot stored as FP16
    are the FP32 ones rounded to nearest, the image is unchanged, and the
    denoised result moves by far less than its error against the reference."""
    hs = P.HostScene.load(scenes.mid_scene(tmp_path / "h", seed=1))
    ctx.upload(hs.pack())
    ctx.build_accel()
    ctx.render(hs.render_params(W, H, 1024, 8, accum_mode=abi.PT_ACCUM_FP32_FP64), stats=False)
    ref = ctx.read_image(fp64=True)
    out = {}
    for name, flags in (("fp32", 0), ("fp16", abi.PT_RENDER_FEATURES_FP16)):
        p = hs.render_params(W, H, 6, 8)
        p.flags = flags
        ctx.render_denoised(trained, p)
        out[name] = (ctx.read_image().copy(), ctx.read_features(), ctx.read_denoised().copy())
    (i32, (a32, n32), d32), (i16, (a16, n16), d16) = out["fp32"], out["fp16"]
    assert np.array_equal(i32.view(np.uint32), i16.view(np.uint32))
    for x32, x16 in ((a32, a16), (n32, n16)):
        assert np.array_equal(x32.astype(np.float16).astype(np.float32), x16)
    e32, e16, shift = meansq(d32, ref), meansq(d16, ref), meansq(d16, d32.astype(np.float64))
    print(f"fp16 features: denoised MSE {e16:.5g} vs fp32 {e32:.5g}; between them {shift:.3g}")
    assert shift < 0.05 * e32 and abs(e16 - e32) < 0.05 * e32
