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
