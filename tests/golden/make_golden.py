"""Generate the golden fixtures of tests/golden/ from the reference itself.

Run here, where the reference tree exists:  python tests/golden/make_golden.py
It needs oracle/_ref (built by `make -C oracle ref` from the reference's own
CPU sources: src/rng.cpp, src/aliastable.h, src/colour.cpp,
src/scene/{camera,lightsample,material}.cpp with the vendored glm, src/io/*
and util/meansq/meansq.cpp) and reads one table from the reference's shader
source as text (shaders/pathtrace/sample.hlsli).  The fixtures let the tests
pin the oracle without the reference tree (it is absent on the GPU machine).
"""
from __future__ import annotations

import base64
import ctypes as C
import json
import re
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

import oracle  # noqa: E402
from pt_gb300 import abi, core, scenes  # noqa: E402

REF = oracle.reference_tree()
if REF is None:
    sys.exit("make_golden: no reference tree (set PT_REFERENCE_TREE)")


def sobol_table():
    text = (REF / "shaders/pathtrace/sample.hlsli").read_text()
    body = text[text.index("directions[SOBOL_MAX_DIMENSION][32]"):]
    body = body[body.index("{") + 1:body.index("};")]
    vals = [int(x, 16) for x in re.findall(r"0x[0-9a-fA-F]+", body)]
    assert len(vals) == 128
    return [vals[32 * d:32 * (d + 1)] for d in range(4)]


def rng_streams(R):
    out = []
    for seed in (0xBD7A0D48, 0, 1, 12345):
        sm = (C.c_uint32 * 4)()
        R.ref_splitmix32_stream(seed, 4, sm)
        u = (C.c_uint32 * 32)()
        f = (C.c_float * 32)()
        R.ref_xshiro128_stream(sm, 32, u, f)
        out.append({"splitmix_seed": seed, "splitmix": list(sm), "xshiro_u32": list(u),
                    "xshiro_f32_bits": [int(np.float32(x).view(np.uint32)) for x in f]})
    return out


def alias_tables(R):
    rng = np.random.default_rng(7)
    cases = [[1.0], [1.0, 1.0], [1.0, 3.0], [0.5, 0.25, 0.25], [10.0, 0.1, 5.0, 0.0, 2.5],
             list(rng.uniform(0, 1, 17).astype(np.float32)), list(rng.lognormal(0, 2, 64).astype(np.float32))]
    out = []
    for w in cases:
        w = np.array(w, np.float32)
        words = (C.c_uint32 * (4 * len(w)))()
        R.ref_alias_build(oracle.fptr(w), len(w), words)
        out.append({"weights_bits": [int(x) for x in w.view(np.uint32)], "bins": list(words)})
    return out


def srgb(R):
    xs = np.concatenate([np.linspace(0, 1, 101), [0.04045, 0.0404, 0.0405, 0.375, 0.45, 0.9, 2.0]]).astype(np.float32)
    return [[int(np.float32(x).view(np.uint32)), int(np.float32(R.ref_from_srgb(float(x))).view(np.uint32))] for x in xs]


CAMERAS = [
    {"position": (-1, 2, -3), "lookdir": (-0.24, -0.06, 0.97), "up": (0, 1, 0), "fov_degrees": 60, "near_plane": 1, "far_plane": 1000,
     "w": 256, "h": 256},
    {"position": (1, -2, 3), "lookdir": (-1, 1.25, -3), "up": (0, 1, 0), "fov_degrees": 60, "near_plane": 0.1, "far_plane": 1000,
     "w": 1024, "h": 1024},
    {"position": (0, -5, 22), "lookdir": (0, 4, -22), "up": (0, 1, 0), "fov_degrees": 45, "near_plane": 0.1, "far_plane": 1000,
     "w": 1920, "h": 1080},
    {"position": (3, 0.5, -7), "lookdir": (0.3, 0.1, 1), "up": (0.1, 1, 0), "fov_degrees": 35, "near_plane": 0.5, "far_plane": 200,
     "w": 640, "h": 480},
]


def cameras(R):
    out = []
    for c in CAMERAS:
        cd = core.camera_struct({k: v for k, v in c.items() if k not in ("w", "h")})
        iv = (C.c_float * 16)()
        ip = (C.c_float * 16)()
        R.ref_camera_params(C.byref(cd), c["w"], c["h"], iv, ip)
        out.append({"camera": c, "inv_view": list(iv), "inv_proj": list(ip)})
    return out


def instance_matrices(R):
    rng = np.random.default_rng(3)
    out = []
    for _ in range(12):
        # random affine transforms built like the .scn t/r/s chain
        A = np.eye(4, dtype=np.float32)
        A[:3, :3] = rng.normal(0, 1, (3, 3)).astype(np.float32)
        A[:3, 3] = rng.uniform(-10, 10, 3).astype(np.float32)
        col = np.ascontiguousarray(A.T.reshape(-1))
        t = (C.c_float * 16)()
        n = (C.c_float * 12)()
        R.ref_instance_matrices(oracle.fptr(col), t, n)
        out.append({"matrix_colmajor": [float(x) for x in col], "transform": list(t), "normal": list(n)})
    return out


LINES = ["t 1 2 3", "t -0.5 0 7.25", "s 2 2 2", "s 0.5 1.5 0.25", "r 1 0 0 3.14", "r 0 1 0 1.5707964", "r 1 1 1 0.3",
         "r 0.2 -0.7 0.1 5.5", "r 0 1 0 -1", "r 0 1 0 0.000001"]


def transforms(R):
    out = []
    for line in LINES:
        m = (C.c_float * 16)()
        rc = R.ref_parse_transform(line.encode(), m)
        out.append({"line": line, "rc": rc, "matrix_colmajor": list(m)})
    return out


def light_scenes():
    """Raw scenes that exercise the light-sampler packing, quirks included."""
    raws = []
    raw, cam = scenes.tiny_raw("two_tris")
    raws.append(("two_tris", raw))
    # instanced emitter (emitter_index per instance vs bins per variant) plus lights
    r2 = {k: (v.copy() if hasattr(v, "copy") else v) for k, v in raw.items()}
    M = np.eye(4, dtype=np.float32)
    M2 = M.copy()
    M2[0, 3] = 3.0
    r2["instance_matrices"] = np.array([M.T.reshape(-1), M.T.reshape(-1), M2.T.reshape(-1)], np.float32)
    r2["mesh_instance_offset"] = np.array([0, 1, 3], np.uint32)
    r2["point_lights"] = np.array([[0, 3, 0, 1, 0.5, 0.25], [2, 1, -1, 4, 4, 4]], np.float32)
    r2["directional_lights"] = np.array([[0, -1, 0.2, 2, 2, 1.5]], np.float32)
    raws.append(("instanced_emitter_and_lights", r2))
    # two emissive meshes with different triangle counts (table-offset quirk)
    p1, n1, uv1, i1 = scenes.icosphere(1)
    p2, n2, uv2, i2 = scenes.quad(1.0, 2.0, True)
    mats = np.array([raw["materials"][1], raw["materials"][1] * np.array([1] * 7 + [3] + [1] * 16, np.float32)], np.float32)
    v = np.concatenate([np.concatenate([p1, n1, uv1], 1), np.concatenate([p2, n2, uv2], 1)]).astype(np.float32)
    r3 = {"vertices": v, "indices": np.concatenate([i1.reshape(-1), i2.reshape(-1)]).astype(np.uint32),
          "meshes": np.array([[0, 0, len(i1), len(p1)], [len(p1), i1.size, len(i2), len(p2)]], np.uint32),
          "mesh_material": np.array([0, 1], np.uint32), "mesh_instance_offset": np.array([0, 1, 2], np.uint32),
          "instance_matrices": np.array([M.T.reshape(-1), M2.T.reshape(-1)], np.float32), "materials": mats,
          "environment_colour": np.zeros(3, np.float32)}
    raws.append(("two_emissive_meshes", r3))
    # an emission-mapped emitter: intensity by the reference's 20-sample estimate
    r4, _ = scenes.textured_raw()
    raws.append(("textured_emitter", r4))
    return raws


def _fixture_raw(raw):
    out = {}
    for k, v in raw.items():
        if k == "textures":
            out[k] = [{"shape": list(img.shape), "srgb": bool(srgb), "data": base64.b64encode(img.tobytes()).decode()}
                      for img, srgb in v]
        else:
            out[k] = np.asarray(v).tolist()
    return out


def light_streams(R):
    out = []
    for name, raw in light_scenes():
        rs, keep = core.raw_to_struct(raw)
        words = (C.c_uint32 * 65536)()
        count = C.c_uint32()
        n = R.ref_light_stream(C.byref(rs), words, 65536, C.byref(count))
        assert n >= 0
        out.append({"name": name, "raw": _fixture_raw(raw),
                    "light_words": list(words[:n]), "light_count": count.value})
    return out


def meansq_cases():
    """MSE of images written by pt_write_hdr as printed by the reference's util/meansq."""
    out = []
    L = abi.lib()
    rng = np.random.default_rng(11)
    with tempfile.TemporaryDirectory() as td:
        for k, (w, h) in enumerate([(8, 8), (13, 7), (24, 16)]):
            a = rng.uniform(0, 4, (h, w, 4)).astype(np.float32)
            b = (a + rng.normal(0, 0.1, a.shape)).clip(0).astype(np.float32)
            pa, pb = f"{td}/a{k}.hdr", f"{td}/b{k}.hdr"
            L.pt_write_hdr(pa.encode(), oracle.fptr(a), w, h)
            L.pt_write_hdr(pb.encode(), oracle.fptr(b), w, h)
            res = subprocess.run([str(oracle.REF_MEANSQ), pa, pb], capture_output=True, text=True, check=True)
            mse = float(res.stdout.strip().split("MSE:")[-1])
            out.append({"w": w, "h": h, "a": base64.b64encode(a.tobytes()).decode(), "b": base64.b64encode(b.tobytes()).decode(),
                        "meansq_stdout_mse": mse, "meansq_stdout": res.stdout})
    return out


def _test_image(w, h, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    a = np.stack([128 + 100 * np.sin(x / 7.0), 128 + 100 * np.cos(y / 5.0 + x / 11.0), x * 255 // max(1, w - 1)], -1)
    a[h // 3:h // 2, w // 4:w // 2] = [250, 10, 30]
    return np.clip(a + rng.normal(0, 12, a.shape), 0, 255).astype(np.uint8)


def jpeg_cases(R):
    """JPEG files and their texels as the reference's stb_image decodes them
    (TextureData, texturedata.cpp:64-76): files written by the reference's
    own stb_image_write (4:2:0 at quality 75, 4:4:4 at 95) and by
    jpeg_writer.py (greyscale, 4:2:2, 4:4:0, 4:2:0 with restart intervals,
    RGB component ids)."""
    import jpeg_writer
    out = []
    for w, h in [(24, 16), (37, 23)]:
        src = _test_image(w, h, w * 7 + h)
        files = []
        for q in (75, 95):
            buf = (C.c_uint8 * (1 << 20))()
            n = R.ref_jpeg_encode(src.ctypes.data_as(C.POINTER(C.c_uint8)), w, h, 3, q, buf, len(buf))
            assert n > 0
            files.append((f"stb_q{q}", bytes(buf[:n])))
        files += [("grey", jpeg_writer.encode(src[..., 0])),
                  ("grey_restart3", jpeg_writer.encode(src[..., 1], restart=3)),
                  ("h2v1", jpeg_writer.encode(src, sampling=(2, 1))),
                  ("h1v2", jpeg_writer.encode(src, sampling=(1, 2))),
                  ("h2v2_restart2", jpeg_writer.encode(src, sampling=(2, 2), restart=2)),
                  ("rgb_ids", jpeg_writer.encode(src, rgb_ids=True))]
        for name, data in files:
            texels = (C.c_uint8 * (w * h * 4))()
            ww, hh, ch = C.c_int(), C.c_int(), C.c_int()
            n = R.ref_image_decode(data, len(data), texels, len(texels), C.byref(ww), C.byref(hh), C.byref(ch))
            assert n == ww.value * hh.value * ch.value
            out.append({"name": f"{name}_{w}x{h}", "jpeg": base64.b64encode(data).decode(), "width": ww.value,
                        "height": hh.value, "channels": ch.value,
                        "stb_texels": base64.b64encode(bytes(texels[:n])).decode()})
    return out


def main():
    only = set(sys.argv[1:])  # fixture file names to write (default: all)
    oracle.build(reference=True)
    R = oracle.ref()
    assert R is not None, "oracle/_ref was not built"
    fixtures = {
        "sobol_table.json": sobol_table(),
        "rng.json": rng_streams(R),
        "alias.json": alias_tables(R),
        "srgb.json": srgb(R),
        "camera.json": cameras(R),
        "instance_matrices.json": instance_matrices(R),
        "parse_transform.json": transforms(R),
        "light_stream.json": light_streams(R),
        "meansq.json": meansq_cases,
        "jpeg.json": lambda: jpeg_cases(R),
    }
    for name, data in fixtures.items():
        if only and name not in only:
            continue
        if callable(data):
            data = data()
        (HERE / name).write_text(json.dumps(data))
        print("wrote", name)


if __name__ == "__main__":
    main()
