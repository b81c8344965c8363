"""Texture sampling of the oracle (CPU): the semantics the CUDA path must
reproduce bit for bit.  The reference samples with Vulkan's linear filter,
REPEAT addressing and level 0 (src/graphics/sampler.cpp:8-22, material.hlsli
SampleLevel(uv, 0)); its hardware's sub-texel weight precision is not
specified, so this build states the filter in float arithmetic: texel centres
at (i + 0.5) / size, weights (1-a)(1-b), a(1-b), (1-a)b, ab.  sRGB textures
(base colour and emission, scene.cpp:42-48) decode each 8-bit value through
the sRGB curve evaluated in double and rounded once."""
import numpy as np
import pytest

import oracle
import pt_gb300 as P
from pt_gb300 import core, scenes


def _scene_with(textures):
    raw, cam = scenes.tiny_raw("two_tris")
    raw["textures"] = textures
    hs = P.HostScene.from_raw(raw, cam)
    return hs, oracle.OracleScene(hs.pack())


def _srgb(c):
    c = c / 255.0
    return np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4).astype(np.float32)


def test_texel_centres_read_texels():
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (5, 7, 4), dtype=np.uint8)
    gray = rng.integers(0, 256, (3, 4), dtype=np.uint8)
    ga = rng.integers(0, 256, (4, 2, 2), dtype=np.uint8)
    hs, o = _scene_with([(img, False), (img, True), (gray, False), (ga, False)])
    for y in range(5):
        for x in range(7):
            u, v = (x + 0.5) / 7, (y + 0.5) / 5
            assert np.array_equal(o.texture_sample(0, u, v), img[y, x] / np.float32(255.0))
            srgb = o.texture_sample(1, u, v)
            assert np.array_equal(srgb[:3], _srgb(img[y, x, :3].astype(np.float64)))
            assert srgb[3] == np.float32(img[y, x, 3]) / np.float32(255.0)
    for y in range(3):
        for x in range(4):
            t = o.texture_sample(2, (x + 0.5) / 4, (y + 0.5) / 3)
            assert np.array_equal(t, np.array([gray[y, x] / np.float32(255.0), 0, 0, 1], np.float32))
    t = o.texture_sample(3, 0.75, 0.125)
    assert np.array_equal(t, np.array([ga[0, 1, 0] / np.float32(255.0), ga[0, 1, 1] / np.float32(255.0), 0, 1], np.float32))


def test_bilinear_weights_and_repeat():
    img = np.zeros((2, 2, 4), np.uint8)
    img[..., 0] = [[0, 255], [51, 102]]
    img[..., 3] = 255
    hs, o = _scene_with([(img, False)])
    # the corner (0, 0) of the texture sits between all four texels (REPEAT wraps the far ones in)
    t = o.texture_sample(0, 0.0, 0.0)
    expect = np.float32(0.25) * (np.float32(0) + np.float32(1.0) + np.float32(0.2) + np.float32(0.4))
    assert abs(t[0] - expect) < 1e-7 and t[3] == 1.0
    # integer shifts of uv sample the same point; negative uv wraps
    for du in (-3.0, -1.0, 1.0, 2.0):
        assert np.array_equal(o.texture_sample(0, 0.25 + du, 0.75), o.texture_sample(0, 0.25, 0.75))
    # a missing texture index reads zero
    assert np.array_equal(o.texture_sample(0 + 7, 0.3, 0.3), np.zeros(4, np.float32))


def test_srgb_table_close_to_reference_curve():
    """The decode table agrees with the reference's own from_srgb
    (colour.cpp, pinned by tests/golden/srgb.json) within float rounding."""
    import json
    from pathlib import Path
    cases = json.loads((Path(__file__).parent / "golden" / "srgb.json").read_text())
    img = np.arange(256, dtype=np.uint8).reshape(16, 16)
    img4 = np.stack([img, img, img, np.full_like(img, 255)], -1)
    hs, o = _scene_with([(img4, True)])
    table = np.array([o.texture_sample(0, ((i % 16) + 0.5) / 16, ((i // 16) + 0.5) / 16)[0] for i in range(256)])
    ref_x = np.array([c[0] for c in cases], np.uint32).view(np.float32)
    ref_y = np.array([c[1] for c in cases], np.uint32).view(np.float32)
    for x, y in zip(ref_x, ref_y):
        k = x * 255.0
        if 0 <= x <= 1 and abs(k - round(k)) < 1e-4:
            assert abs(table[int(round(k))] - y) <= 2e-7 + 1e-6 * y
