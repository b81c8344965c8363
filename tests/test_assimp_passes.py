"""The Assimp post-processing the reference asks for on every model file
(scene.cpp:537-550), as the scene front end restates it (assimp_post.cpp):
RemoveRedundantMaterials, FindInstances, OptimizeGraph, OptimizeMeshes,
FindDegenerates, JoinIdenticalVertices.  Assimp 5.4.3 is not in the
reference tree, so these tests check the restated behaviour on hand-built
files: what each pass keeps, merges and moves, and that the world-space
geometry the renderer sees is unchanged."""
import json
from pathlib import Path

import numpy as np
import pytest

import pt_gb300 as P
from pt_gb300 import scenes


def _scn(d: Path, model: str) -> Path:
    p = d / "s.scn"
    p.write_text(f"camera:\n\nobjects:\nm {model}\nm\n")
    return p


def _gltf(d: Path, meshes, nodes, roots, materials, extra=None) -> Path:
    """meshes: list of lists of primitives (positions (n,3), indices (m,) or
    None, material); one buffer, normals +y, uvs from x/z."""
    blob, views, acc = bytearray(), [], []

    def add(arr, comp, typ):
        arr = np.ascontiguousarray(arr)
        views.append({"buffer": 0, "byteOffset": len(blob), "byteLength": arr.nbytes})
        blob.extend(arr.tobytes())
        blob.extend(b"\0" * ((4 - arr.nbytes % 4) % 4))
        acc.append({"bufferView": len(views) - 1, "componentType": comp, "count": len(arr), "type": typ})
        return len(acc) - 1

    jm = []
    for prims in meshes:
        jp = []
        for pos, idx, mat in prims:
            pos = np.asarray(pos, np.float32)
            nrm = np.tile(np.float32([0, 1, 0]), (len(pos), 1))
            uv = pos[:, [0, 2]].copy()
            prim = {"attributes": {"POSITION": add(pos, 5126, "VEC3"), "NORMAL": add(nrm, 5126, "VEC3"),
                                   "TEXCOORD_0": add(uv, 5126, "VEC2")}, "material": mat}
            if idx is not None:
                prim["indices"] = add(np.asarray(idx, np.uint32), 5125, "SCALAR")
            jp.append(prim)
        jm.append({"primitives": jp})
    (d / "m.bin").write_bytes(bytes(blob))
    doc = {"asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": roots}], "nodes": nodes, "meshes": jm,
           "materials": materials, "accessors": acc, "bufferViews": views,
           "buffers": [{"uri": "m.bin", "byteLength": len(blob)}]}
    if extra:
        doc.update(extra)
    (d / "m.gltf").write_text(json.dumps(doc))
    return _scn(d, "m.gltf")


def _mat(r, g=0.5, b=0.5, rough=0.5):
    return {"pbrMetallicRoughness": {"baseColorFactor": [r, g, b, 1.0], "roughnessFactor": rough, "metallicFactor": 0.0}}


QUAD = np.float32([[0, 0, 0], [1, 0, 0], [1, 0, 1], [0, 0, 1]])
QUAD_IDX = [0, 1, 2, 0, 2, 3]
TRI = np.float32([[0, 1, 0], [1, 1, 0], [0, 1, 1]])


def _world_triangles(raw) -> np.ndarray:
    """Every instanced triangle in world space, sorted (a set to compare)."""
    out = []
    v = raw["vertices"]
    for m, (vo, io, tris, _) in enumerate(raw["meshes"]):
        idx = raw["indices"][io:io + 3 * tris].reshape(-1, 3) + vo
        for j in range(raw["mesh_instance_offset"][m], raw["mesh_instance_offset"][m + 1]):
            M = raw["instance_matrices"][j].reshape(4, 4).T.astype(np.float64)
            p = (v[idx.reshape(-1), :3].astype(np.float64) @ M[:3, :3].T + M[:3, 3]).round(4).reshape(-1, 3, 3)
            for tri in p:  # each triangle's corners in lexicographic order
                out.append(tri[np.lexsort(tri.T[::-1])].reshape(9))
    a = np.array(out)
    return a[np.lexsort(a.T[::-1])]


def test_redundant_materials_are_merged_and_unused_removed(tmp_path):
    """Materials 0 and 2 are equal (merged), 1 is unused (dropped); the two
    primitives of material 0/2 in one node then merge into one mesh."""
    path = _gltf(tmp_path, [[(QUAD, QUAD_IDX, 0), (QUAD + 2, QUAD_IDX, 2), (TRI, None, 3)]], [{"mesh": 0}], [0],
                 [_mat(0.2), _mat(0.9), _mat(0.2), _mat(0.4)])
    raw = P.HostScene.load(path).raw()
    assert len(raw["materials"]) == 2
    assert sorted(raw["mesh_material"].tolist()) == [0, 1]
    assert len(raw["meshes"]) == 2 and sorted(raw["meshes"][:, 2].tolist()) == [1, 4]
    merged = [k for k in range(2) if raw["meshes"][k, 2] == 4][0]
    # the absorbed primitive's triangles come first, the absorbing one's last
    vo, io = raw["meshes"][merged, 0], raw["meshes"][merged, 1]
    first = raw["vertices"][vo + raw["indices"][io], :3]
    assert np.array_equal(first, QUAD[0] + 2)


def test_identical_meshes_become_instances(tmp_path):
    """Two glTF meshes with equal data and material under two nodes: one mesh,
    two instances (FindInstances), left instanced by the graph passes."""
    path = _gltf(tmp_path, [[(QUAD, QUAD_IDX, 0)], [(QUAD, QUAD_IDX, 0)]],
                 [{"mesh": 0, "translation": [0, 0, 0]}, {"mesh": 1, "translation": [3, 0, 0]}], [0, 1], [_mat(0.3)])
    raw = P.HostScene.load(path).raw()
    assert len(raw["meshes"]) == 1
    assert raw["instance_matrices"].shape == (2, 16)
    assert sorted(raw["instance_matrices"][:, 12].tolist()) == [0.0, 3.0]


def test_graph_is_flattened_and_meshes_joined_into_one_space(tmp_path):
    """root(T) -> a(R, mesh 0) -> b(S, mesh 1): both meshes used once, so the
    graph collapses to one node holding both meshes in b's space; one mesh
    per material remains and the world-space triangles are unchanged."""
    q = [0.0, 0.38268343, 0.0, 0.9238795]
    nodes = [{"children": [1], "translation": [1.0, 2.0, 3.0]},
             {"mesh": 0, "rotation": q, "children": [2]},
             {"mesh": 1, "scale": [2.0, 0.5, 2.0], "translation": [0.5, 0.0, 0.0]}]
    before = _world_triangles({
        "vertices": np.concatenate([np.c_[QUAD, np.zeros((4, 5), np.float32)], np.c_[TRI, np.zeros((3, 5), np.float32)]]),
        "indices": np.uint32(QUAD_IDX + [0, 1, 2]), "meshes": np.array([[0, 0, 2, 4], [4, 6, 1, 3]]),
        "mesh_instance_offset": [0, 1, 2], "instance_matrices": None} | {"instance_matrices": _chain(nodes)})
    path = _gltf(tmp_path, [[(QUAD, QUAD_IDX, 0)], [(TRI, None, 0)]], nodes, [0], [_mat(0.3)])
    raw = P.HostScene.load(path).raw()
    assert len(raw["meshes"]) == 1 and raw["meshes"][0, 2] == 3 and raw["instance_matrices"].shape == (1, 16)
    np.testing.assert_allclose(_world_triangles(raw), before, atol=2e-4)


def _chain(nodes):
    """Instance matrices of nodes[1] and nodes[2] composed root to leaf in float64."""
    def local(n):
        M = np.eye(4)
        if "rotation" in n:
            x, y, z, w = n["rotation"]
            M[:3, :3] = [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                         [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                         [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]
        S = np.diag(n.get("scale", [1, 1, 1]) + [1])
        T = np.eye(4)
        T[:3, 3] = n.get("translation", [0, 0, 0])
        return T @ M @ S
    a = local(nodes[0]) @ local(nodes[1])
    b = a @ local(nodes[2])
    return np.array([a.T.reshape(-1), b.T.reshape(-1)], np.float32)


def test_nodes_with_lights_stay_in_place(tmp_path):
    """A node carrying a KHR_lights_punctual light is locked: the graph pass
    keeps it and its child; their meshes are not joined across it."""
    nodes = [{"children": [1, 2]}, {"mesh": 0, "translation": [2, 0, 0]},
             {"extensions": {"KHR_lights_punctual": {"light": 0}}, "children": [3], "translation": [0, 5, 0]},
             {"mesh": 1, "translation": [-2, 0, 0]}]
    extra = {"extensions": {"KHR_lights_punctual": {"lights": [{"type": "point", "intensity": 2.0}]}}}
    path = _gltf(tmp_path, [[(QUAD, QUAD_IDX, 0)], [(TRI, None, 1)]], nodes, [0], [_mat(0.3), _mat(0.6)], extra)
    raw = P.HostScene.load(path).raw()
    assert len(raw["meshes"]) == 2
    m = raw["instance_matrices"].reshape(-1, 4, 4)
    assert sorted(tuple(x[3, :3]) for x in m) == [(-2.0, 5.0, 0.0), (2.0, 0.0, 0.0)]
    assert raw["point_lights"].shape == (1, 6)


def test_degenerate_triangles_become_zero_triangles(tmp_path):
    """A triangle with two equal vertex positions keeps fewer indices under
    FindDegenerates' defaults; the reference stores it as (0, 0, 0)."""
    pos = np.float32([[0, 0, 0], [1, 0, 0], [1, 0, 1], [1, 0, 0]])
    path = _gltf(tmp_path, [[(pos, [0, 1, 2, 1, 3, 2], 0)]], [{"mesh": 0}], [0], [_mat(0.3)])
    raw = P.HostScene.load(path).raw()
    idx = raw["indices"].reshape(-1, 3)
    assert idx.shape == (2, 3) and idx[1].tolist() == [0, 0, 0] and idx[0].tolist() == [0, 1, 2]
    assert raw["meshes"][0, 3] == 3  # vertex 3 repeats vertex 1 and is joined


def test_identical_vertices_are_joined_and_unused_dropped(tmp_path):
    """A non-indexed primitive (every corner its own vertex) keeps one vertex
    per distinct corner; a vertex no triangle uses is dropped."""
    corners = QUAD[[0, 1, 2, 0, 2, 3]]
    path = _gltf(tmp_path, [[(corners, None, 0)]], [{"mesh": 0}], [0], [_mat(0.3)])
    raw = P.HostScene.load(path).raw()
    assert raw["meshes"][0, 3] == 4 and raw["indices"].tolist() == [0, 1, 2, 0, 2, 3]
    pos = np.concatenate([QUAD, [[9, 9, 9]]]).astype(np.float32)
    path = _gltf(tmp_path, [[(pos, QUAD_IDX, 0)]], [{"mesh": 0}], [0], [_mat(0.3)])
    raw = P.HostScene.load(path).raw()
    assert raw["meshes"][0, 3] == 4


def test_obj_groups_with_one_material_merge(tmp_path):
    """OBJ groups are nodes under one root with identity transforms: the graph
    pass joins them and meshes of the same material merge (absorbed ones
    first), while another material stays its own mesh."""
    (tmp_path / "m.mtl").write_text("newmtl a\nKd 0.5 0.5 0.5\nnewmtl b\nKd 0.2 0.2 0.2\n")
    (tmp_path / "o.obj").write_text(
        "mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 1 0 1\nv 0 0 1\nv 5 0 5\n"
        "g one\nusemtl a\nf 1 2 3\ng two\nusemtl b\nf 1 3 4\ng three\nusemtl a\nf 2 5 3\n")
    raw = P.HostScene.load(_scn(tmp_path, "o.obj")).raw()
    assert len(raw["meshes"]) == 2 and raw["meshes"][:, 2].tolist() == [2, 1]
    vo, io = raw["meshes"][0, :2]
    first = raw["vertices"][vo + raw["indices"][io:io + 3], :3]
    assert np.array_equal(first, np.float32([[1, 0, 0], [5, 0, 5], [1, 0, 1]]))  # group three's triangle first


def test_instanced_mesh_with_material_split(tmp_path):
    """A glTF mesh used by two nodes keeps its own mesh per primitive and both
    instances; a singly used mesh next to it is unaffected."""
    nodes = [{"mesh": 0}, {"mesh": 0, "translation": [0, 0, 4]}, {"mesh": 1, "translation": [4, 0, 0]}]
    path = _gltf(tmp_path, [[(QUAD, QUAD_IDX, 0), (TRI, None, 1)], [(TRI, None, 0)]], nodes, [0, 1, 2],
                 [_mat(0.3), _mat(0.7)])
    raw = P.HostScene.load(path).raw()
    inst = np.diff(raw["mesh_instance_offset"]).tolist()
    assert sorted(inst) == [1, 2, 2] and len(raw["meshes"]) == 3


def test_generated_benchmark_scenes_are_unchanged_in_geometry(tmp_path):
    """One mesh, node and material per file: the passes only join identical
    vertices, so the world-space triangles stay those of the files."""
    raw = P.HostScene.load(scenes.small_scene(tmp_path, seed=0)).raw()
    from oracle import scn_reader
    rr, _ = scn_reader.read_scn(tmp_path / "small.scn")
    for k in ("vertices", "indices", "meshes", "instance_matrices"):
        assert np.array_equal(np.asarray(raw[k]), np.asarray(rr[k])), k
