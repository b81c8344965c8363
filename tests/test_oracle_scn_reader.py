"""The oracle's own .scn + glTF reader (oracle/scn_reader.py) against the
product's scene front end (pt_scene_load): the same raw scene, bit for bit,
and the same packed device view and camera.  The reader is what the
reference arm of the benchmark uses, so that arm never loads libptgpu.so."""
import numpy as np
import pytest

import oracle
import pt_gb300 as P
from oracle import scn_reader
from pt_gb300 import abi, scenes

KEYS = ("vertices", "indices", "meshes", "mesh_material", "mesh_instance_offset", "instance_matrices", "materials",
        "environment_colour")


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape:
        return False
    if a.dtype == np.float32:
        return np.array_equal(a.view(np.uint32), b.view(np.uint32))
    return np.array_equal(a, b)


@pytest.mark.parametrize("make", [scenes.small_scene, scenes.mid_scene], ids=["small", "mid"])
def test_reader_equals_product_loader(tmp_path, make):
    path = make(tmp_path)
    raw, cam = scn_reader.read_scn(path)
    hs = P.HostScene.load(path)
    want = hs.raw()
    for k in KEYS:
        assert _same(raw[k], want[k]), k
    cd = hs.camera()
    for k in ("position", "lookdir", "up"):
        assert list(getattr(cd, k)) == [float(x) for x in cam[k]], k
    for k in ("fov_degrees", "near_plane", "far_plane", "focus_dist", "lens_radius", "exposure"):
        assert getattr(cd, k) == float(cam[k]), k
    # packed by the oracle's packer from the reader's arrays = packed by the product
    rs, keep = scn_reader.raw_struct(raw)
    packed = oracle.OraclePacked(rs)
    a, b = P.view_arrays(hs.pack()), P.view_arrays(packed.view)
    for k in a:
        if isinstance(a[k], np.ndarray):
            assert np.array_equal(a[k], b[k]), k
        else:
            assert a[k] == b[k], k
    # camera matrices through the oracle equal the product's
    p_or = abi.RenderParams()
    oracle.lib().or_camera_params(scn_reader.camera_desc(cam), 64, 48, p_or)
    p_pt = hs.render_params(64, 48, 1, 1)
    assert bytes(p_or.inv_view) == bytes(p_pt.inv_view) and bytes(p_or.inv_proj) == bytes(p_pt.inv_proj)


def test_raw_struct_of_generated_raw_scenes():
    """The oracle's marshalling of the generators' raw scenes (which carry no
    light arrays): the oracle's packing equals the product's, on the heavy
    configuration's scene."""
    raw, cam = scenes.heavy_scene()
    rs, keep = scn_reader.raw_struct(raw)
    packed = oracle.OraclePacked(rs)
    hs = P.HostScene.from_raw(raw, cam)  # the packed view borrows its memory
    a = P.view_arrays(hs.pack())
    b = P.view_arrays(packed.view)
    for k in a:
        if isinstance(a[k], np.ndarray):
            assert np.array_equal(a[k], b[k]), k
        else:
            assert a[k] == b[k], k
