"""Precision study: the error each reduced-precision choice adds, against
the FP64 reference, per scene configuration.

  * accumulation: the FP32 running mean (the reference's arithmetic) against
    FP64 sums of the same samples;
  * feature storage: denoiser features and half-sample snapshot stored as
    FP16 (PT_RENDER_FEATURES_FP16) against FP32;
  * the network in BF16 (BF16 weights, activations and gradients, FP32
    accumulation) against the same network evaluated in FP64 by the oracle
    (oracle/unet_oracle.py) on a 128x128 crop of the denoiser input.

Each row prints one JSON line ("precision ..."); errors are meansq over RGB
(util/meansq) in radiance units, next to the error of the result itself
against the converged FP64 reference, so the added error can be read as a
fraction of the total.
"""
import json

import numpy as np
import pytest

import oracle.unet_oracle as UO
import pt_gb300 as P
from pt_gb300 import abi, scenes
from pt_gb300.denoise import WEIGHTS_DIR, UNet, load_params

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CROP = 128
DENOISE_SPP = 6


def meansq(a, b):
    d = a[..., :3].astype(np.float64) - b[..., :3].astype(np.float64)
    return float(np.sum(d * d) / (d.size - 1))


def _configs(tmp_path):
    small = P.HostScene.load(scenes.small_scene(tmp_path / "s", seed=0))
    mid = P.HostScene.load(scenes.mid_scene(tmp_path / "m", seed=1))
    raw, cam = scenes.heavy_scene()
    heavy = P.HostScene.from_raw(raw, cam)
    # (name, scene, width, height, bounces, rr_start, reference spp)
    return [("small", small, 256, 256, 8, 1, 4096), ("mid", mid, 512, 512, 8, 1, 2048),
            ("heavy", heavy, 480, 272, 12, 4, 1024)]


@pytest.fixture(scope="module")
def params():
    w = WEIGHTS_DIR / "unet.bin"
    if not w.exists():
        pytest.fail(f"trained weights missing: {w}")
    return load_params(w)


def test_precision_per_config(tmp_path, params):
    ctx = P.Context(0)
    rows = []
    for name, hs, W, H, B, rr, ref_spp in _configs(tmp_path):
        view = hs.pack()
        ctx.upload(view)
        ctx.build_accel()
        ctx.render(hs.render_params(W, H, ref_spp, B, rr_start=rr, accum_mode=abi.PT_ACCUM_FP32_FP64), stats=False)
        ref = ctx.read_image(fp64=True)
        row = {"config": name, "size": [W, H], "bounces": B, "reference_spp": ref_spp}
        # accumulation: FP32 running mean vs FP64 sums of the same samples
        for spp in (DENOISE_SPP, 64):
            ctx.render(hs.render_params(W, H, spp, B, rr_start=rr, accum_mode=abi.PT_ACCUM_FP32_FP64), stats=False)
            m32, m64 = ctx.read_image(), ctx.read_image(fp64=True)
            row[f"plain_{spp}spp"] = {"mse_vs_ref": meansq(m32, ref), "fp32_vs_fp64_accumulation": meansq(m32, m64)}
            assert row[f"plain_{spp}spp"]["fp32_vs_fp64_accumulation"] < 1e-6 * row[f"plain_{spp}spp"]["mse_vs_ref"]
        # feature storage: FP16 vs FP32, through the whole denoised pipeline
        net = UNet(1, H, W)
        net.set_params(params)
        den = {}
        for tag, flags in (("fp32", 0), ("fp16", abi.PT_RENDER_FEATURES_FP16)):
            p = hs.render_params(W, H, DENOISE_SPP, B, rr_start=rr)
            p.flags = flags
            ctx.render_denoised(net, p)
            den[tag] = ctx.read_denoised().copy()
        row["denoised_6spp"] = {"mse_vs_ref_fp32_features": meansq(den["fp32"], ref),
                                "mse_vs_ref_fp16_features": meansq(den["fp16"], ref),
                                "fp16_vs_fp32_features": meansq(den["fp16"], den["fp32"])}
        assert row["denoised_6spp"]["fp16_vs_fp32_features"] < 0.05 * row["denoised_6spp"]["mse_vs_ref_fp32_features"]
        # the network in BF16 vs FP64, on a centre crop of the 6-spp input (FP32 features)
        p = hs.render_params(W, H, DENOISE_SPP, B, rr_start=rr)
        ctx.render_noisy(p)
        ctx.denoise_input(DENOISE_SPP, net.input_ptr, int(abi.lib().pt_unet_base(net.handle)))
        y0, x0 = (H - CROP) // 2, (W - CROP) // 2
        x_full = net.input_tensor()[0, y0:y0 + CROP, x0:x0 + CROP].clone()
        b_full = net.base_tensor()[0, y0:y0 + CROP, x0:x0 + CROP].clone()
        crop = UNet(1, CROP, CROP)
        crop.set_params(params)
        crop.input_tensor()[0].copy_(x_full)
        crop.base_tensor()[0].copy_(b_full)
        crop.forward()
        torch.cuda.synchronize()
        y_gpu = crop.output_tensor()[0].cpu().numpy().astype(np.float64)
        x64 = x_full.float().cpu().numpy().astype(np.float64)[None]
        y64, _ = UO.forward(params.astype(np.float64), x64, base=b_full.cpu().numpy().astype(np.float64)[None])
        lin = lambda y: np.expm1(np.maximum(y[..., :3], 0.0))  # noqa: E731
        ref_crop = ref[y0:y0 + CROP, x0:x0 + CROP]
        row["network_crop"] = {"crop": [CROP, CROP], "bf16_vs_fp64_network": meansq(lin(y_gpu), lin(y64[0])),
                               "mse_vs_ref_bf16_network": meansq(lin(y_gpu), ref_crop),
                               "mse_vs_ref_fp64_network": meansq(lin(y64[0]), ref_crop)}
        assert row["network_crop"]["bf16_vs_fp64_network"] < 0.5 * row["network_crop"]["mse_vs_ref_fp64_network"]
        crop.close()
        net.close()
        rows.append(row)
        print("precision " + json.dumps(row))
    ctx.close()
