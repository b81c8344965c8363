"""Failure detection without a GPU fault: malformed scene data is rejected
on the host before any kernel sees it, degenerate but valid scenes render,
and a traversal that reaches its iteration cap stops and reports
PT_ERR_TIMEOUT (the cap is lowered in a child process with
PT_TRAVERSAL_CAP, read once per process), after which the GPU still works."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import oracle
import pt_gb300 as P
from pt_gb300 import abi, scenes

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def ctx():
    c = P.Context(0)
    yield c
    c.close()


def _upload_error(ctx, raw):
    hs = P.HostScene.from_raw(raw, None)
    with pytest.raises(P.PtError) as e:
        ctx.upload(hs.pack())
    return e.value


def _tiny():
    raw, cam = scenes.tiny_raw("two_tris")
    return {k: (v.copy() if hasattr(v, "copy") else v) for k, v in raw.items()}, cam


def test_non_finite_vertex_is_rejected(ctx):
    raw, _ = _tiny()
    raw["vertices"][2, 1] = np.nan
    e = _upload_error(ctx, raw)
    assert e.status == abi.PT_ERR_INVALID and "non-finite" in str(e)
    raw["vertices"][2, 1] = np.inf
    assert _upload_error(ctx, raw).status == abi.PT_ERR_INVALID


def test_malformed_views_are_rejected(ctx):
    raw, cam = _tiny()
    hs = P.HostScene.from_raw(raw, cam)  # owns the arrays the view points to
    view = hs.pack()
    arr = P.view_arrays(view)
    # an index outside its mesh, through a raw view (the host packer would refuse it first)
    idx = arr["indices"].copy()
    idx[0] = 1000
    keep = [idx]
    v2 = abi.SceneView.from_buffer_copy(view)
    v2.indices = idx.ctypes.data_as(abi.C.POINTER(abi.C.c_uint32))
    with pytest.raises(P.PtError) as e:
        ctx.upload(v2)
    assert e.value.status == abi.PT_ERR_INVALID and "index outside" in str(e.value)
    # an instance naming a missing material
    inst = arr["instances"].copy().reshape(-1, 32)
    inst[0, 3] = 99
    keep.append(inst)
    v3 = abi.SceneView.from_buffer_copy(view)
    v3.instances = inst.ctypes.data_as(abi.C.POINTER(abi.InstanceData))
    with pytest.raises(P.PtError) as e:
        ctx.upload(v3)
    assert e.value.status == abi.PT_ERR_INVALID and "material" in str(e.value)
    del keep


def test_empty_and_zero_triangle_scenes_render(ctx):
    raw, cam = _tiny()
    # a mesh without triangles, instanced, next to a normal one
    raw["meshes"] = np.concatenate([raw["meshes"], np.array([[0, 0, 0, 0]], np.uint32)])
    raw["mesh_material"] = np.concatenate([raw["mesh_material"], np.array([0], np.uint32)])
    raw["mesh_instance_offset"] = np.concatenate([raw["mesh_instance_offset"], [raw["mesh_instance_offset"][-1] + 1]]).astype(np.uint32)
    raw["instance_matrices"] = np.concatenate([raw["instance_matrices"], np.eye(4, dtype=np.float32).reshape(1, 16)])
    hs = P.HostScene.from_raw(raw, cam)
    view = hs.pack()
    ctx.upload(view)
    ctx.build_accel()
    p = hs.render_params(24, 16, 2, 3)
    st = ctx.render(p)
    assert st.error_word == 0
    ref, _ = oracle.OracleScene(view).render(p)
    assert np.array_equal(ctx.read_image().view(np.uint32), ref.view(np.uint32))
    # no instances at all: every pixel sees the environment colour
    empty = {k: v for k, v in raw.items()}
    empty["mesh_instance_offset"] = np.zeros_like(raw["mesh_instance_offset"])
    empty["instance_matrices"] = np.zeros((0, 16), np.float32)
    hs2 = P.HostScene.from_raw(empty, cam)
    ctx.upload(hs2.pack())
    ctx.build_accel()
    ctx.render(hs2.render_params(8, 8, 1, 2))
    img = ctx.read_image()
    assert np.allclose(img[..., :3], np.asarray(raw["environment_colour"], np.float32))


_CHECKED = """
import sys, numpy as np
import pt_gb300 as P
from pt_gb300 import abi, scenes
assert abi.LIB_PATH.name == "libptgpu_checked.so"
hs = P.HostScene.load(scenes.small_scene(__import__("pathlib").Path(sys.argv[1]), seed=0))
ctx = P.Context(0)
ctx.upload(hs.pack())
ctx.build_accel()
p = hs.render_params(64, 48, 3, 6)
st = ctx.render(p)
assert st.error_word == 0
np.save(sys.argv[2], ctx.read_image())
# an out-of-range child link in the traversed TLAS root: caught before any access
assert abi.lib().pt_debug_poke_tlas_link(ctx._h, 0x7FFF0000) == abi.PT_OK
try:
    ctx.render(p)
    print("no error")
except P.PtError as e:
    print("status", e.status, str(e))
ctx.build_accel()  # repaired by a rebuild
ctx.render(p)
np.save(sys.argv[3], ctx.read_image())
"""


def test_checked_build_matches_and_catches_bad_indices(ctx, tmp_path):
    """The bounds-checked library (PT_CHECKED=1 selects it; set in a child)
    renders the same image as the normal one, and a corrupted BVH link is
    reported as PT_ERR_DEVICE "index out of range" instead of being followed;
    the normal build refuses the fault injection."""
    a, b = tmp_path / "a.npy", tmp_path / "b.npy"
    r = subprocess.run([sys.executable, "-c", _CHECKED, str(tmp_path / "scene"), str(a), str(b)],
                       env=dict(os.environ, PT_CHECKED="1"), cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert f"status {abi.PT_ERR_DEVICE}" in r.stdout and "index out of range" in r.stdout, r.stdout
    hs = P.HostScene.load(scenes.small_scene(tmp_path / "scene2", seed=0))
    ctx.upload(hs.pack())
    ctx.build_accel()
    ctx.render(hs.render_params(64, 48, 3, 6))
    want = ctx.read_image()
    assert np.array_equal(np.load(a).view(np.uint32), want.view(np.uint32))
    assert np.array_equal(np.load(b).view(np.uint32), want.view(np.uint32))
    assert abi.lib().pt_debug_poke_tlas_link(ctx._h, 0x7FFF0000) == abi.PT_ERR_UNSUPPORTED


_CAPPED = """
import pt_gb300 as P
from pt_gb300 import abi, scenes
raw, cam = scenes.tiny_raw("two_tris")
hs = P.HostScene.from_raw(raw, cam)
ctx = P.Context(0)
ctx.upload(hs.pack())
ctx.build_accel()
try:
    ctx.render(hs.render_params(16, 16, 1, 2))
    print("no error")
except P.PtError as e:
    print("status", e.status)
"""


def test_watchdog_reports_timeout_and_gpu_stays_usable(ctx):
    env = dict(os.environ, PT_TRAVERSAL_CAP="2")
    r = subprocess.run([sys.executable, "-c", _CAPPED], env=env, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert f"status {abi.PT_ERR_TIMEOUT}" in r.stdout, r.stdout
    # this process (no cap) still renders
    raw, cam = _tiny()
    hs = P.HostScene.from_raw(raw, cam)
    ctx.upload(hs.pack())
    ctx.build_accel()
    assert ctx.render(hs.render_params(8, 8, 1, 2)).error_word == 0
