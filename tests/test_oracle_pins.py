"""Pins of the oracle (and of the product's host pieces) against the reference.

The fixtures in tests/golden/ come from the reference's own CPU code compiled
from its sources (tests/golden/make_golden.py).  When the reference's build is
present (oracle/_ref) the same checks also run live against it.
"""
import base64
import ctypes as C
import json
import tempfile
from pathlib import Path

import numpy as np
import pytest

import oracle
import pt_gb300 as P
from pt_gb300 import abi, core, scenes

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name):
    return json.loads((GOLDEN / name).read_text())


def test_sobol_table_matches_reference_shader():
    table = load("sobol_table.json")
    L = oracle.lib()
    for d in range(4):
        for b in range(32):
            assert L.or_sobol(1 << b, d) == table[d][b], (d, b)


def test_sobol_linearity():
    L = oracle.lib()
    rng = np.random.default_rng(0)
    for _ in range(200):
        a, b = (int(x) for x in rng.integers(0, 2**32, 2, dtype=np.uint64))
        for d in range(4):
            assert L.or_sobol(a ^ b, d) == L.or_sobol(a, d) ^ L.or_sobol(b, d)


def test_host_rng_matches_reference():
    L = oracle.lib()
    for case in load("rng.json"):
        sm = (C.c_uint32 * 4)()
        L.or_splitmix32_stream(case["splitmix_seed"], 4, sm)
        assert list(sm) == case["splitmix"]
        u = (C.c_uint32 * 32)()
        f = (C.c_float * 32)()
        L.or_xshiro128_stream(sm, 32, u, f)
        assert list(u) == case["xshiro_u32"]
        assert [int(np.float32(x).view(np.uint32)) for x in f] == case["xshiro_f32_bits"]

def test_emitter_intensity_stream_known_answer():
    """lightsample.cpp:45-46 constructs Xshiro128(seeder.next() x 4); GCC
    evaluates the four arguments right to left, so the state is the four
    Splitmix32 outputs in reverse.  Known answer of that stream."""
    L = oracle.lib()
    sm = (C.c_uint32 * 4)()
    L.or_splitmix32_stream(0xBD7A0D48, 4, sm)
    rev = (C.c_uint32 * 4)(*list(sm)[::-1])
    u = (C.c_uint32 * 4)()
    f = (C.c_float * 4)()
    L.or_xshiro128_stream(rev, 4, u, f)
    assert list(u)[:3] == [4170722718, 3171359881, 1779237160]
    assert abs(f[3] - 0.580254376) < 1e-8


def test_scene_rng_matches_reference():
    case = load("rng.json")[0]
    L = oracle.lib()
    sm = (C.c_uint32 * 4)()
    L.or_splitmix32_stream(case["splitmix_seed"], 4, sm)
    rev = (C.c_uint32 * 4)(*list(sm)[::-1])
    u = (C.c_uint32 * 32)()
    L.or_xshiro128_stream(rev, 32, u, None)
    r = scenes.SceneRng(case["splitmix_seed"])
    assert [r.next() for _ in range(32)] == list(u)


def test_alias_tables_match_reference():
    L = oracle.lib()
    for case in load("alias.json"):
        w = np.array(case["weights_bits"], np.uint32).view(np.float32)
        n = len(w)
        p = np.zeros(n, np.float32)
        q = np.zeros(n, np.float32)
        a = np.zeros(n, np.uint32)
        L.or_alias_build(oracle.fptr(w), n, oracle.fptr(p), oracle.fptr(q), oracle.uptr(a))
        bins = np.array(case["bins"], np.uint32).reshape(n, 4)
        assert np.array_equal(p.view(np.uint32), bins[:, 0])
        assert np.array_equal(q.view(np.uint32), bins[:, 1])
        assert np.array_equal(a, bins[:, 2])


def test_from_srgb_matches_reference():
    L = oracle.lib()
    for xb, yb in load("srgb.json"):
        x = float(np.uint32(xb).view(np.float32))
        assert np.float32(L.or_from_srgb(x)).view(np.uint32) == yb
        assert np.float32(abi.lib().pt_from_srgb(x)).view(np.uint32) == yb


@pytest.mark.parametrize("which", ["oracle", "product"])
def test_camera_matrices_match_reference(which):
    """The reference rounds every step of the glm chain in float; oracle and
    product evaluate it in FP64 and round once.  They agree to a few ulps."""
    for case in load("camera.json"):
        c = case["camera"]
        cd = core.camera_struct({k: v for k, v in c.items() if k not in ("w", "h")})
        p = abi.RenderParams()
        if which == "oracle":
            oracle.lib().or_camera_params(C.byref(cd), c["w"], c["h"], C.byref(p))
        else:
            assert abi.lib().pt_camera_params(C.byref(cd), c["w"], c["h"], C.byref(p)) == 0
        iv = np.array(list(p.inv_view), np.float32)
        ip = np.array(list(p.inv_proj), np.float32)
        riv = np.array(case["inv_view"], np.float32)
        rip = np.array(case["inv_proj"], np.float32)
        # rows 0-2 are what the ray generation reads
        np.testing.assert_allclose(iv[:12], riv[:12], rtol=3e-6, atol=3e-7)
        np.testing.assert_allclose(ip[:12], rip[:12], rtol=3e-6, atol=3e-7)


def test_instance_normal_matrix_matches_reference():
    """InstanceData.transform is bit-exact; the normal matrix (glm float
    inverse in the reference, FP64 inverse here) agrees to a few ulps."""
    for case in load("instance_matrices.json"):
        col = np.array(case["matrix_colmajor"], np.float32)
        raw, _ = scenes.tiny_raw("two_tris")
        raw["instance_matrices"] = np.stack([col, np.eye(4, dtype=np.float32).reshape(-1)])
        rs, keep = core.raw_to_struct(raw)
        pk = oracle.OraclePacked(rs)
        arr = P.view_arrays(pk.view)
        inst = arr["instances"].reshape(-1, 32)[0]
        t = inst[4:20].view(np.float32)
        n = inst[20:32].view(np.float32)
        assert np.array_equal(t, np.array(case["transform"], np.float32))
        rn = np.array(case["normal"], np.float32)
        np.testing.assert_allclose(n, rn, rtol=2e-5, atol=2e-6)


def _write_one_object_scene(d: Path, lines):
    scenes.write_gltf(d / "obj.gltf", scenes.quad(1.0, 0.0, False), {"base": (0.5, 0.5, 0.5)})
    text = "camera:\nposition 0 0 0\n\nobjects:\nobj obj.gltf\n\nobj\n" + "\n".join(lines) + "\n"
    (d / "one.scn").write_text(text)
    return d / "one.scn"


def test_scn_transforms_match_reference_parser():
    for case in load("parse_transform.json"):
        with tempfile.TemporaryDirectory() as td:
            hs = P.HostScene.load(_write_one_object_scene(Path(td), [case["line"]]))
            m = hs.raw()["instance_matrices"][0]
            assert np.array_equal(m, np.array(case["matrix_colmajor"], np.float32)), case["line"]


def _raw_from_fixture(r):
    raw = {}
    for k, v in r.items():
        if k == "textures":
            raw[k] = [(np.frombuffer(base64.b64decode(t["data"]), np.uint8).reshape(t["shape"]), t["srgb"]) for t in v]
            continue
        dt = np.uint32 if k in ("indices", "meshes", "mesh_material", "mesh_instance_offset") else np.float32
        raw[k] = np.array(v, dt)
    return raw


@pytest.mark.parametrize("which", ["oracle", "product"])
def test_light_streams_match_reference(which):
    for case in load("light_stream.json"):
        raw = _raw_from_fixture(case["raw"])
        if which == "oracle":
            rs, keep = core.raw_to_struct(raw)
            pk = oracle.OraclePacked(rs)
            view = pk.view
        else:
            hs = P.HostScene.from_raw(raw)
            view = hs.pack()
        arr = P.view_arrays(view)
        assert arr["light"].tolist() == case["light_words"], case["name"]
        assert arr["light_count"] == case["light_count"]


def test_meansq_matches_reference_tool():
    L = abi.lib()
    for case in load("meansq.json"):
        w, h = case["w"], case["h"]
        a = np.frombuffer(base64.b64decode(case["a"]), np.float32).reshape(h, w, 4)
        b = np.frombuffer(base64.b64decode(case["b"]), np.float32).reshape(h, w, 4)
        with tempfile.TemporaryDirectory() as td:
            imgs = []
            for name, img in (("a", a), ("b", b)):
                path = f"{td}/{name}.hdr".encode()
                assert L.pt_write_hdr(path, oracle.fptr(np.ascontiguousarray(img)), w, h) == 0
                ptr = C.POINTER(C.c_float)()
                W, H = C.c_uint32(), C.c_uint32()
                assert L.pt_read_hdr(path, C.byref(ptr), C.byref(W), C.byref(H)) == 0
                imgs.append(np.ctypeslib.as_array(ptr, shape=(h, w, 4)).copy())
                L.pt_host_free(ptr)
        mse = oracle.meansq(imgs[0], imgs[1])
        # meansq prints 6 significant digits
        assert abs(mse - case["meansq_stdout_mse"]) <= 5e-6 * abs(case["meansq_stdout_mse"]) + 1e-12


def test_live_reference_when_available():
    R = oracle.ref()
    if R is None:
        pytest.skip("reference build (oracle/_ref) not present on this machine")
    L = oracle.lib()
    rng = np.random.default_rng(5)
    for _ in range(50):
        w = rng.lognormal(0, 1.5, int(rng.integers(1, 40))).astype(np.float32)
        n = len(w)
        words = (C.c_uint32 * (4 * n))()
        R.ref_alias_build(oracle.fptr(w), n, words)
        p = np.zeros(n, np.float32)
        q = np.zeros(n, np.float32)
        a = np.zeros(n, np.uint32)
        L.or_alias_build(oracle.fptr(w), n, oracle.fptr(p), oracle.fptr(q), oracle.uptr(a))
        bins = np.array(list(words), np.uint32).reshape(n, 4)
        assert np.array_equal(p.view(np.uint32), bins[:, 0]) and np.array_equal(q.view(np.uint32), bins[:, 1])
        assert np.array_equal(a, bins[:, 2])
