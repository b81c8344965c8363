"""The host-side scene front end and the `pt` CLI argument handling (no GPU).

Mirrors the reference's .scn grammar (scenebuild.cpp:132-365), its error
messages, the glTF import rules of this build and main.cpp's argument checks.
"""
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
import pt_gb300 as P
from pt_gb300 import abi, core, scenes
from pt_gb300.build import CLI


def write_obj(d: Path, name="obj", **mat):
    scenes.write_gltf(d / f"{name}.gltf", scenes.quad(1.0, 0.0, False), mat or {"base": (0.5, 0.5, 0.5)})


def scn(d: Path, text: str) -> Path:
    p = d / "s.scn"
    p.write_text(text)
    return p


def load_error(path) -> str:
    with pytest.raises(P.PtError) as e:
        P.HostScene.load(path)
    return str(e.value)


def test_camera_defaults_and_fields(tmp_path):
    write_obj(tmp_path)
    hs = P.HostScene.load(scn(tmp_path, "camera:\n\nobjects:\nobj obj.gltf\nobj\n"))
    c = hs.camera()
    assert list(c.position) == [0, 0, 0] and list(c.lookdir) == [0, 0, -1] and list(c.up) == [0, 1, 0]
    assert (c.fov_degrees, c.exposure) == (45.0, 1.0)
    assert abs(c.near_plane - 0.1) < 1e-7 and c.far_plane == 1000.0
    hs = P.HostScene.load(scn(tmp_path, "camera:\nposition 1 2 3\nfov 60\nexposure 10\nfocusdist 8\nlensradius 0.03\n"
                                        "envcol 0.375 0.45 0.9\nnear 1\n\nobjects:\nobj obj.gltf\nobj\n"))
    c = hs.camera()
    assert list(c.position) == [1, 2, 3] and c.fov_degrees == 60 and c.exposure == 10
    assert abs(c.focus_dist - 8) < 1e-7 and abs(c.lens_radius - 0.03) < 1e-7 and c.near_plane == 1.0
    env = hs.raw()["environment_colour"]
    assert np.array_equal(env, np.array([abi.lib().pt_from_srgb(x) for x in (0.375, 0.45, 0.9)], np.float32))


def test_tabs_and_carriage_returns_are_removed(tmp_path):
    write_obj(tmp_path)
    hs = P.HostScene.load(scn(tmp_path, "camera:\r\nposition 1\t 2 3\r\n\nobjects:\r\nobj obj.gltf\r\nobj\r\nt 1 0 0\r\n"))
    assert list(hs.camera().position) == [1, 2, 3]
    assert hs.raw()["instance_matrices"][0][12] == 1.0


@pytest.mark.parametrize("text,message", [
    ("objects:\nobj obj.gltf\nobj\n", "No camera section in scene description."),
    ("camera:\ncamera:\n", "Camera already set."),
    ("camera:\nbogus 1\n", "Unrecognised token in camera section bogus"),
    ("nonsense\n", "Unrecognised token nonsense"),
    ("camera:\n\nobjects:\nt 1 2 3\n", "No instance to translate."),
    ("camera:\n\nobjects:\nobj obj.gltf\nobj\nt 1 2\n", "Translation did not have three coordinates"),
    ("camera:\n\nobjects:\nobj obj.gltf\nobj\nr 1 0 0\n", "Rotation did not have three coordinates and angle"),
    ("camera:\n\nobjects:\nobj obj.gltf\nobj\nr 0 0 0 1\n", "Rotation axis was (close to) zero"),
    ("camera:\n\nobjects:\nmissing\n", "Object missing not recognised."),
    ("camera:\n\nobjects:\nplight 1 2 3 , 1 1\n", "Invalid light syntax."),
    ("camera:\nposition 1 2\n", "Vectors need three components"),
    ("camera:\n\nobjects:\nobj nothere.gltf\nobj\n", "Could not open file"),
])
def test_scn_errors(tmp_path, text, message):
    write_obj(tmp_path)
    assert message in load_error(scn(tmp_path, text))


def test_transform_order_and_identity_rotation(tmp_path):
    """t/r/s lines pre-multiply (scenebuild.cpp:210-221); angle < 1e-5 (also
    negative) gives the identity (lalgebra.cpp:21-22)."""
    write_obj(tmp_path)
    hs = P.HostScene.load(scn(tmp_path, "camera:\n\nobjects:\nobj obj.gltf\nobj\ns 2 2 2\nt 1 0 0\nobj\nr 0 1 0 -1\nobj\n"))
    m = hs.raw()["instance_matrices"].reshape(-1, 4, 4)  # column-major rows = columns
    np.testing.assert_array_equal(m[0].T, np.array([[2, 0, 0, 1], [0, 2, 0, 0], [0, 0, 2, 0], [0, 0, 0, 1]], np.float32))
    np.testing.assert_array_equal(m[1], np.eye(4, dtype=np.float32))
    np.testing.assert_array_equal(m[2], np.eye(4, dtype=np.float32))


def test_lights_and_ignored_material_tokens(tmp_path):
    write_obj(tmp_path)
    hs = P.HostScene.load(scn(tmp_path, "camera:\n\nobjects:\nobj obj.gltf\nobj\nbasecol 1 0 0\nroughness 0.1\n"
                                        "plight 0 3 0 , 1 1 1\ndlight 0 -1 0 , 0.5 0.5 0.5\n"))
    raw = hs.raw()
    assert raw["point_lights"].shape == (1, 6) and raw["directional_lights"].shape == (1, 6)
    assert raw["point_lights"][0][3] == 1.0
    view = hs.pack()
    assert view.light_count == 2


def test_subscene_instances_multiply_and_materials_copy(tmp_path):
    """scenebuild.cpp:309-362: meshes/materials appended per subscene,
    instances = scene instances x object instances; unused objects skipped."""
    write_obj(tmp_path, "a")
    write_obj(tmp_path, "b", base=(0.1, 0.2, 0.3), emission_strength=4.0)
    write_obj(tmp_path, "c")
    hs = P.HostScene.load(scn(tmp_path, "camera:\n\nobjects:\na a.gltf\nb b.gltf\nc c.gltf\n\na\nb\nt 0 1 0\na\n"))
    raw = hs.raw()
    assert raw["mesh_material"].tolist() == [0, 1]
    assert raw["mesh_instance_offset"].tolist() == [0, 2, 3]
    mats = raw["materials"]
    assert mats[1][7] == 4.0 and mats[1][4] == 1.0  # emission (1,1,1) x strength 4
    details = hs.details()
    assert "2 meshes" in details and "3 instances" in details and "1 instances with emission" in details


def test_gltf_defaults_uv_flip_and_nodes(tmp_path):
    p, n, uv, idx = scenes.quad(2.0, 0.0, False)
    uv = np.array([[0.1, 0.1], [0.9, 0.1], [0.9, 0.7], [0.1, 0.7]], np.float32)
    scenes.write_gltf(tmp_path / "q.gltf", (p, n, uv, idx), {"base": (1, 1, 1)})
    doc = json.loads((tmp_path / "q.gltf").read_text())
    del doc["materials"][0]["pbrMetallicRoughness"]["metallicFactor"]
    doc["nodes"] = [{"children": [1], "translation": [0, 2, 0]}, {"mesh": 0, "scale": [2, 2, 2]}]
    (tmp_path / "q.gltf").write_text(json.dumps(doc))
    hs = P.HostScene.load(scn(tmp_path, "camera:\n\nobjects:\nq q.gltf\nq\n"))
    raw = hs.raw()
    v = raw["vertices"]
    expect_v = np.float32(1.0) - (np.float32(1.0) - uv[:, 1])
    assert np.array_equal(v[:, 7], expect_v)  # Assimp flips v twice
    m = raw["instance_matrices"][0].reshape(4, 4).T
    np.testing.assert_array_equal(m, np.array([[2, 0, 0, 0], [0, 2, 0, 2], [0, 0, 2, 0], [0, 0, 0, 1]], np.float32))
    mat = raw["materials"][0]
    assert mat[9] == 1.0  # glTF default metallic factor as Assimp reports it
    assert mat[12:15].tolist() == [0.5, 0.5, 0.5] and mat[21] == 0.5


def test_pack_matches_oracle_on_mid_scene(tmp_path):
    hs = P.HostScene.load(scenes.mid_scene(tmp_path, seed=1))
    a = P.view_arrays(hs.pack())
    rs, keep = core.raw_to_struct(hs.raw())
    packed = oracle.OraclePacked(rs)  # keeps the packed arrays alive
    b = P.view_arrays(packed.view)
    for k in a:
        if isinstance(a[k], np.ndarray):
            assert np.array_equal(a[k], b[k]), k
        else:
            assert a[k] == b[k], k
    assert a["light_count"] == 32


def run_cli(*args):
    return subprocess.run([str(CLI), *map(str, args)], capture_output=True, text=True, timeout=60)


@pytest.mark.parametrize("args,message", [
    ([], "Error: Expected path to scene."),
    (["a.scn", "b.scn"], "Error: Unexpected number of arguments."),
    (["--headless", "x.scn"], "Error: No output file was given (required for headless execution)."),
    (["--headless", "-o", "x.png", "-s", "0", "x.scn"], "Error: Invalid sample count: 0."),
    (["--headless", "-o", "x.png", "-b", "-1", "x.scn"], "Error: Invalid number of ray bounces: -1."),
    (["--headless", "-o", "x.png", "-w", "0", "x.scn"], "Error: Invalid dimensions: (0, 400)."),
    (["--headless", "-o", "x.png", "-f", "jpg", "x.scn"], "Error: Output format is invalid: jpg"),
    (["--bogus", "x.scn"], "Error: Unknown option --bogus."),
    (["-s"], "Error: Option -s has no value."),
    (["--headless", "-o", "x.png", "-sabc", "x.scn"], "was not an integer: abc"),
    (["--headless", "-o", "x.png", "missing.scn"], "Error: Could not open file missing.scn"),
])
def test_cli_argument_errors(args, message):
    r = run_cli(*args)
    assert r.returncode == 1
    assert message in r.stderr


def test_cli_help():
    r = run_cli("--help")
    assert r.returncode == 0 and r.stdout.startswith("Usage: ") and "--samples, -s" in r.stdout


def _textured_gltf(d: Path, name: str, images, textures, materials, prim_material=0):
    """A quad glTF whose document carries the given images / textures /
    materials; prim_material is the primitive's material, or a list: one
    primitive (the same quad) per material listed."""
    scenes.write_gltf(d / f"{name}.gltf", scenes.quad(2.0, 0.0, False), {"base": (1, 1, 1)})
    doc = json.loads((d / f"{name}.gltf").read_text())
    doc["images"] = images
    doc["textures"] = textures
    doc["materials"] = materials
    prim = doc["meshes"][0]["primitives"][0]
    mats = prim_material if isinstance(prim_material, list) else [prim_material]
    doc["meshes"][0]["primitives"] = [dict(prim, material=m) for m in mats]
    (d / f"{name}.gltf").write_text(json.dumps(doc))


def _u32(f):
    return int(np.float32(f).view(np.uint32))


def test_gltf_texture_order_srgb_channels_and_transparency(tmp_path):
    """Texture indices follow first use over the materials, in the order
    base colour, emission, metallic-roughness, normal (process_texture,
    scene.cpp:50-72); the first use decides sRGB; 3-channel images are stored
    as 4; a base-colour map with alpha below one makes the material
    transparent (scene.cpp:344-355)."""
    rng = np.random.default_rng(3)
    rgb = rng.integers(0, 256, (5, 7, 3), dtype=np.uint8)
    gray = rng.integers(0, 256, (4, 4), dtype=np.uint8)
    ga = rng.integers(0, 256, (3, 6, 2), dtype=np.uint8)
    rgba = rng.integers(0, 256, (6, 5, 4), dtype=np.uint8)
    rgba[..., 3] = 255
    rgba[2, 3, 3] = 254
    for n, img in (("rgb", rgb), ("gray", gray), ("ga", ga), ("rgba", rgba)):
        (tmp_path / f"{n}.png").write_bytes(scenes.png_bytes(img))
    images = [{"uri": "rgba.png"}, {"uri": "rgb.png"}, {"uri": "gray.png"}, {"uri": "ga.png"}, {"uri": "rgb.png"}]
    textures = [{"source": i} for i in range(5)]
    materials = [
        {"pbrMetallicRoughness": {"baseColorTexture": {"index": 1}, "metallicRoughnessTexture": {"index": 2}},
         "normalTexture": {"index": 4}},
        {"pbrMetallicRoughness": {"baseColorTexture": {"index": 3}}, "emissiveTexture": {"index": 0}},
        {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}}},
    ]
    _textured_gltf(tmp_path, "tq", images, textures, materials, prim_material=[0, 1, 2])
    hs = P.HostScene.load(scn(tmp_path, "camera:\n\nobjects:\ntq tq.gltf\ntq\n"))
    raw = hs.raw()
    tex = raw["textures"]
    # rgb.png (base of material 0) -> 0, gray.png -> 1, rgb.png again (normal, same uri) -> 0,
    # ga.png (base of material 1) -> 2, rgba.png (emission) -> 3
    assert len(tex) == 4
    assert tex[0][0].shape == (5, 7, 4) and tex[0][1] is True
    assert np.array_equal(tex[0][0][..., :3], rgb) and np.all(tex[0][0][..., 3] == 255)
    assert tex[1][0].shape == (4, 4) and tex[1][1] is False and np.array_equal(tex[1][0], gray)
    assert tex[2][0].shape == (3, 6, 2) and tex[2][1] is False  # sRGB only exists for 4 channels
    assert np.array_equal(tex[3][0], rgba) and tex[3][1] is True
    m = raw["materials"]
    bits = [_u32(r[11]) for r in m]
    assert bits[0] == abi.PT_BASE_COLOUR_MAP_BIT | abi.PT_ROUGHNESS_METALNESS_MAP_BIT | abi.PT_NORMAL_MAP_BIT
    assert (_u32(m[0][0]), _u32(m[0][8]), _u32(m[0][10])) == (0, 1, 0)
    assert bits[1] == abi.PT_BASE_COLOUR_MAP_BIT | abi.PT_EMISSION_MAP_BIT  # 2-channel map: no transparency
    assert (_u32(m[1][0]), _u32(m[1][4])) == (2, 3)
    assert bits[2] == abi.PT_BASE_COLOUR_MAP_BIT | abi.PT_MATERIAL_IS_TRANSPARENT_BIT and _u32(m[2][0]) == 3
    assert "4 textures" in hs.details()


def test_gltf_texture_offsets_across_objects(tmp_path):
    """A second object's textures follow the first's and its map indices move
    by the same offset, except the specular and sheen maps, whose offset lands
    in the unused .w slot (offset_maps_by, material.cpp:16-42)."""
    rng = np.random.default_rng(4)
    for n in ("a", "b", "c"):
        (tmp_path / f"{n}.png").write_bytes(scenes.png_bytes(rng.integers(0, 256, (2, 3, 4), dtype=np.uint8)))
    _textured_gltf(tmp_path, "one", [{"uri": "a.png"}], [{"source": 0}],
                   [{"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}}}])
    mat = {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}},
           "extensions": {"KHR_materials_specular": {"specularColorTexture": {"index": 1}},
                          "KHR_materials_sheen": {"sheenColorTexture": {"index": 0}}}}
    _textured_gltf(tmp_path, "two", [{"uri": "b.png"}, {"uri": "c.png"}], [{"source": 0}, {"source": 1}], [mat])
    hs = P.HostScene.load(scn(tmp_path, "camera:\n\nobjects:\none one.gltf\ntwo two.gltf\none\ntwo\n"))
    raw = hs.raw()
    assert len(raw["textures"]) == 3
    m = raw["materials"]
    assert _u32(m[0][0]) == 0
    assert _u32(m[1][0]) == 1  # base colour: local 0 + offset 1
    assert _u32(m[1][12]) == 1 and _u32(m[1][15]) == 1  # specular: .x keeps local 1, .w gets the offset
    assert _u32(m[1][16]) == 0 and _u32(m[1][19]) == 1  # sheen: .x keeps local 0


def test_jpeg_textures_are_rejected(tmp_path):
    (tmp_path / "j.jpg").write_bytes(b"\xff\xd8\xff\xe0" + bytes(64))
    _textured_gltf(tmp_path, "j", [{"uri": "j.jpg"}], [{"source": 0}],
                   [{"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}}}])
    msg = load_error(scn(tmp_path, "camera:\n\nobjects:\njq j.gltf\njq\n"))
    assert "JPEG" in msg


def test_textured_pack_matches_oracle():
    raw, cam = scenes.textured_raw()
    hs = P.HostScene.from_raw(raw, cam)
    a = P.view_arrays(hs.pack())
    rs, keep = core.raw_to_struct(raw)
    packed = oracle.OraclePacked(rs)
    b = P.view_arrays(packed.view)
    for k in a:
        if isinstance(a[k], np.ndarray):
            assert np.array_equal(a[k], b[k]), k
        else:
            assert a[k] == b[k], k
    assert a["textures"].size == 6 * len(raw["textures"]) and a["texels"].size == sum(t.size for t, _ in raw["textures"])


def _bits(f):
    return int(np.float32(f).view(np.uint32))


def test_obj_import(tmp_path):
    """Wavefront OBJ + MTL with the reference's Assimp material keys: one
    mesh per object/group/material run, fan triangulation, negative indices,
    v flipped, flat normals where faces have none, Kd/Ke sRGB-decoded, d as
    opacity (transparency bit), Pr/Pm factors, maps in first-use order."""
    (tmp_path / "rm.png").write_bytes(scenes.png_bytes(np.full((2, 2, 4), 200, np.uint8)))
    (tmp_path / "kd.png").write_bytes(scenes.png_bytes(np.full((2, 2, 3), 90, np.uint8)))
    (tmp_path / "m.mtl").write_text(
        "newmtl red\nKd 0.5 0.25 0.125\nd 0.5\nPr 0.3\nPm 1\n"
        "newmtl glow\nKd 0 0 0\nKe 1 0.5 0\n"
        "newmtl tex\nmap_Kd kd.png\nmap_Pr rm.png\nmap_Pm rm.png\n")
    (tmp_path / "o.obj").write_text(
        "mtllib m.mtl\n"
        "v 0 0 0\nv 1 0 0\nv 1 0 1\nv 0 0 1\n"
        "vt 0 0\nvt 1 0\nvt 1 0.25\nvt 0 1\n"
        "vn 0 1 0\n"
        "f 1/1 2/2 3/3 4/4\n"           # default material, quad -> 2 triangles, flat normals
        "usemtl red\nf -4//1 -3//1 -2//1\n"  # negative indices, given normal
        "o second\nusemtl glow\nf 1 3 2\n"
        "usemtl tex\nf 1/1 2/2 3/3\n")
    hs = P.HostScene.load(scn(tmp_path, "camera:\n\nobjects:\nob o.obj\nob\n"))
    raw = hs.raw()
    meshes = raw["meshes"]
    assert meshes.shape[0] == 4 and meshes[:, 2].tolist() == [2, 1, 1, 1]
    v = raw["vertices"]
    # per-corner vertices joined by JoinIdenticalVertices: the quad keeps 4
    assert meshes[0, 3] == 4
    tri = raw["indices"][meshes[0, 1]:meshes[0, 1] + 6].reshape(2, 3) + meshes[0, 0]
    first = v[tri.reshape(-1)]
    assert np.allclose(first[:, 3:6], [0, -1, 0]) or np.allclose(first[:, 3:6], [0, 1, 0])
    assert np.allclose(first[:3, 7], [1, 1, 0.75])  # 1 - v
    assert np.array_equal(first[3:, 0:3], np.array([[0, 0, 0], [1, 0, 1], [0, 0, 1]], np.float32))  # fan (0, 2, 3)
    mats = raw["materials"]
    mm = raw["mesh_material"]
    default, red, glow, tex = (mats[i] for i in mm)
    assert np.allclose(default[0:4], [P.abi.lib().pt_from_srgb(0.6)] * 3 + [1.0])
    assert red[0] == np.float32(P.abi.lib().pt_from_srgb(0.5)) and red[3] == 0.5
    assert (_bits(red[11]) & abi.PT_MATERIAL_IS_TRANSPARENT_BIT) and red[8] == np.float32(0.3) and red[9] == 1.0
    assert glow[4] == 1.0 and glow[5] == np.float32(P.abi.lib().pt_from_srgb(0.5)) and glow[7] == 1.0
    tb = _bits(tex[11])
    assert tb & abi.PT_BASE_COLOUR_MAP_BIT and tb & abi.PT_ROUGHNESS_METALNESS_MAP_BIT
    assert (_bits(tex[0]), _bits(tex[8])) == (0, 1)
    t = raw["textures"]
    assert len(t) == 2 and t[0][1] is True and t[0][0].shape == (2, 2, 4) and t[1][1] is False
    assert "2 textures" in hs.details()


def test_obj_errors(tmp_path):
    (tmp_path / "bad.obj").write_text("v 0 0 0\nf 1 2 3\n")
    assert "missing position" in load_error(scn(tmp_path, "camera:\n\nobjects:\nb bad.obj\nb\n"))
