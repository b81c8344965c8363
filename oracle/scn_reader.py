"""The oracle's own reader of the drop-in scene formats: a `.scn` description
(camera section + objects section) and the glTF 2.0 objects it names, turned
into the raw in-memory scene (the arrays of pt_raw_scene) and the camera
description, with no call into the product library.

TEST INFRASTRUCTURE ONLY: a second, independent restatement of the
reference's scene import, used by bench.py's reference arm (which must not
load libptgpu.so) and checked against the product's loader by
tests/test_oracle_scn_reader.py.  It covers what the benchmark scenes use:
camera keys, envcol, objects, instances with s/r/t transforms, glTF meshes
(POSITION, NORMAL, TEXCOORD_0, indices, node TRS/matrix hierarchy) and
factor materials (base colour, metallic/roughness, emission with
KHR_materials_emissive_strength, KHR_materials_transmission), one mesh,
node and material per model file, and the reference's Assimp
post-processing where it acts on such a file (FindDegenerates,
JoinIdenticalVertices).  Textures, point/directional lights, OBJ files and
multi-mesh files are refused.

Reference semantics followed (file:line in anveba/pt):
  .scn camera section            src/scene/scenebuild.cpp:132-197 (defaults :138-144)
  objects section, s/r/t order   src/scene/scenebuild.cpp:200-262 (new transform
                                 multiplies from the left, :213-221)
  translation/rotation/scaling   src/lalgebra.cpp:5-94 (rotation is the identity
                                 for angle < 1e-5, :21)
  instance = scene x object      src/scene/scenebuild.cpp:340-352
  sRGB decode of colours         src/colour.cpp:12-14 (double arithmetic)
  glTF material factors          src/scene/scene.cpp:74-296 via Assimp's glTF
                                 importer (base colour and emission factors
                                 sRGB-decoded, :94, :134; emissive strength
                                 :140-143; opacity = 1 - transmission :96-108;
                                 specular 0.5 :227; clearcoat roughness 0.5)
  UV flip round trip             Assimp glTF importer + aiProcess_FlipUVs
                                 (scene.cpp:537-550): v stored as 1 - (1 - v)
All float arithmetic is done in float32 in the order the C++ evaluates it;
cos/sin of a float angle come from the host C library's cosf/sinf, the
functions std::cos/std::sin of a float call in the C++.
"""
from __future__ import annotations

import base64
import ctypes as C
import ctypes.util as ctypes_util
import json
import math
from pathlib import Path

import numpy as np

F = np.float32
_LIBM = C.CDLL(ctypes_util.find_library("m") or "libm.so.6")
_LIBM.cosf.restype = _LIBM.sinf.restype = C.c_float
_LIBM.cosf.argtypes = _LIBM.sinf.argtypes = [C.c_float]
BASE_COLOUR_MAP_BIT = 1 << 0
MATERIAL_IS_TRANSPARENT_BIT = 1 << 13


def _mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """glm column-major product a*b (m[col][row]), each entry summed left to right in float32."""
    r = np.zeros((4, 4), np.float32)
    for j in range(4):
        for i in range(4):
            r[j, i] = ((a[0, i] * b[j, 0] + a[1, i] * b[j, 1]) + a[2, i] * b[j, 2]) + a[3, i] * b[j, 3]
    return r


def _translation(x, y, z):
    r = np.eye(4, dtype=np.float32)
    r[3, 0:3] = (x, y, z)
    return r


def _scaling(x, y, z):
    r = np.zeros((4, 4), np.float32)
    r[0, 0], r[1, 1], r[2, 2], r[3, 3] = x, y, z, F(1)
    return r


def _rotation(ux, uy, uz, angle):
    """lalgebra.cpp:16-55 in float32."""
    if float(angle) < 1e-5:
        return np.eye(4, dtype=np.float32)
    ln = np.sqrt(F((ux * ux + uy * uy) + uz * uz))
    if float(ln) < 1e-5:
        raise ValueError("Rotation axis was (close to) zero")
    inv = F(F(1) / ln)
    ux, uy, uz = F(ux * inv), F(uy * inv), F(uz * inv)
    c = F(_LIBM.cosf(float(angle)))
    s = F(_LIBM.sinf(float(angle)))
    one = F(1)
    r = np.zeros((4, 4), np.float32)
    r[0, 0] = ux * ux + (one - ux * ux) * c
    r[0, 1] = uy * ux * (one - c) + uz * s
    r[0, 2] = uz * ux * (one - c) - uy * s
    r[1, 0] = ux * uy * (one - c) - uz * s
    r[1, 1] = uy * uy + (one - uy * uy) * c
    r[1, 2] = uz * uy * (one - c) + ux * s
    r[2, 0] = ux * uz * (one - c) + uy * s
    r[2, 1] = uy * uz * (one - c) - ux * s
    r[2, 2] = uz * uz + (one - uz * uz) * c
    r[3, 3] = one
    return r


def from_srgb(x) -> np.float32:
    """colour.cpp:12-14: double arithmetic, float result."""
    x = float(F(x))
    return F(x / 12.92 if x <= 0.04045 else math.pow((x + 0.055) / 1.055, 2.4))


def _tokens(line: str):
    return [t for t in line.split(" ") if t]


def _stof(s: str) -> np.float32:
    return F(float(s))


def read_gltf(path: Path):
    """One glTF 2.0 file -> (vertices (n,8), indices, meshes [(voff, ioff, tris, verts)],
    mesh_material, mesh_instances [[4x4 column-major]], materials (k,24))."""
    doc = json.loads(Path(path).read_text())
    folder = Path(path).parent
    buffers = []
    for b in doc.get("buffers", []):
        uri = b["uri"]
        if uri.startswith("data:"):
            buffers.append(base64.b64decode(uri[uri.index(",") + 1:]))
        else:
            buffers.append((folder / uri).read_bytes())
    if doc.get("textures") or doc.get("images"):
        raise NotImplementedError("the oracle's scene reader does not load textures")

    def accessor(i):
        a = doc["accessors"][i]
        bv = doc["bufferViews"][a["bufferView"]]
        comp = {5126: np.float32, 5125: np.uint32, 5123: np.uint16, 5121: np.uint8}[a["componentType"]]
        if a.get("normalized"):
            raise NotImplementedError("normalized accessors")
        n = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4}[a["type"]]
        off = bv.get("byteOffset", 0) + a.get("byteOffset", 0)
        size = np.dtype(comp).itemsize
        stride = bv.get("byteStride", 0) or size * n
        raw = np.frombuffer(buffers[bv["buffer"]], np.uint8)
        rows = [raw[off + k * stride: off + k * stride + size * n].view(comp) for k in range(a["count"])] \
            if stride != size * n else [raw[off: off + a["count"] * size * n].view(comp)]
        return np.concatenate(rows).reshape(a["count"], n)

    materials = []
    for m in doc.get("materials", []):
        pbr = m.get("pbrMetallicRoughness", {})
        ext = m.get("extensions", {})
        if any(k in pbr for k in ("baseColorTexture", "metallicRoughnessTexture")) or \
                any(k in m for k in ("emissiveTexture", "normalTexture")):
            raise NotImplementedError("textured materials")
        row = np.zeros(24, np.float32)
        bcf = pbr.get("baseColorFactor", [1.0, 1.0, 1.0, 1.0])
        opacity = F(1)
        if "KHR_materials_transmission" in ext:
            opacity = F(F(1) - F(ext["KHR_materials_transmission"].get("transmissionFactor", 0.0)))
        row[0:3] = [from_srgb(F(bcf[k])) for k in range(3)]
        row[3] = opacity
        ef = m.get("emissiveFactor", [0.0, 0.0, 0.0])
        row[4:7] = [from_srgb(F(ef[k])) for k in range(3)]
        row[7] = F(ext["KHR_materials_emissive_strength"].get("emissiveStrength", 1.0)) \
            if "KHR_materials_emissive_strength" in ext else F(1)
        row[8] = F(pbr.get("roughnessFactor", 1.0))
        row[9] = F(pbr.get("metallicFactor", 1.0))
        row[12:15] = F(0.5)
        row[21] = F(0.5)
        bits = 0
        if row[3] < 1:  # has_transparency (scene.cpp:344-355)
            bits |= MATERIAL_IS_TRANSPARENT_BIT
        row[11] = np.uint32(bits).view(np.float32)
        materials.append(row)

    verts, idxs, meshes, mesh_mat, prims_of = [], [], [], [], []
    vcount = icount = 0
    for mesh in doc["meshes"]:
        prims_of.append([])
        for p in mesh["primitives"]:
            if p.get("mode", 4) != 4:
                continue
            at = p["attributes"]
            pos = accessor(at["POSITION"]).astype(np.float32)
            if "NORMAL" not in at:
                raise NotImplementedError("generated normals")
            nrm = accessor(at["NORMAL"]).astype(np.float32)
            if "TEXCOORD_0" in at:
                uv = accessor(at["TEXCOORD_0"]).astype(np.float32)
                v = (F(1) - (F(1) - uv[:, 1])).astype(np.float32)
                uv = np.stack([uv[:, 0], v], 1)
            else:
                uv = np.zeros((len(pos), 2), np.float32)
            idx = accessor(p["indices"]).reshape(-1).astype(np.uint32) if "indices" in p \
                else np.arange(len(pos), dtype=np.uint32)
            idx = idx[: len(idx) // 3 * 3]
            if idx.size and idx.max() >= len(pos):
                raise ValueError("index outside the vertex range")
            verts.append(np.concatenate([pos, nrm, uv], 1).astype(np.float32))
            idxs.append(idx)
            prims_of[-1].append(len(meshes))
            meshes.append((vcount, icount, len(idx) // 3, len(pos)))
            vcount += len(pos)
            icount += len(idx)
            mat = p.get("material", -1)
            if mat < 0:
                raise NotImplementedError("primitives without a material")
            mesh_mat.append(mat)

    def node_matrix(n):
        if "matrix" in n:
            return np.array(n["matrix"], np.float32).reshape(4, 4)
        t = [F(x) for x in n.get("translation", [0, 0, 0])]
        qx, qy, qz, qw = [F(x) for x in n.get("rotation", [0, 0, 0, 1])]
        s = [F(x) for x in n.get("scale", [1, 1, 1])]
        one, two = F(1), F(2)
        R = np.eye(4, dtype=np.float32)
        R[0, 0] = one - two * (qy * qy + qz * qz)
        R[0, 1] = two * (qx * qy + qz * qw)
        R[0, 2] = two * (qx * qz - qy * qw)
        R[1, 0] = two * (qx * qy - qz * qw)
        R[1, 1] = one - two * (qx * qx + qz * qz)
        R[1, 2] = two * (qy * qz + qx * qw)
        R[2, 0] = two * (qx * qz + qy * qw)
        R[2, 1] = two * (qy * qz - qx * qw)
        R[2, 2] = one - two * (qx * qx + qy * qy)
        return _mul(_mul(_translation(*t), R), _scaling(*s))

    mesh_instances = [[] for _ in meshes]
    stack = [(r, np.eye(4, dtype=np.float32)) for r in doc["scenes"][doc.get("scene", 0)]["nodes"]]
    while stack:
        ni, parent = stack.pop()
        n = doc["nodes"][ni]
        M = _mul(parent, node_matrix(n))
        if "mesh" in n:
            for m in prims_of[n["mesh"]]:
                mesh_instances[m].append(M)
        for c in reversed(n.get("children", [])):
            stack.append((c, M))
    return (np.concatenate(verts) if verts else np.zeros((0, 8), np.float32),
            np.concatenate(idxs) if idxs else np.zeros(0, np.uint32), meshes, mesh_mat, mesh_instances,
            np.array(materials, np.float32).reshape(-1, 24))


def assimp_single_mesh(v: np.ndarray, idx: np.ndarray):
    """The reference's Assimp post-processing (scene.cpp:537-550) where it
    acts on a file of one mesh, one node and one material: FindDegenerates
    with Assimp's defaults (a triangle with two equal vertex positions keeps
    fewer indices; the reference stores it as (0, 0, 0)), then
    JoinIdenticalVertices (vertices no face uses dropped, vertices equal in
    every attribute to an earlier one replaced by it, first occurrence in
    vertex order kept).  Returns (vertices, indices)."""
    f = idx.reshape(-1, 3).astype(np.int64)
    p = v[:, :3]
    faces = []  # the indices each face keeps
    for a, b, c in f:
        keep = [a, b, c]
        i = 0
        while i < len(keep):
            k = i + 1
            while k < len(keep):
                if np.array_equal(p[keep[i]], p[keep[k]]):
                    del keep[k]
                else:
                    k += 1
            i += 1
        faces.append(keep)
    used = np.zeros(len(v), bool)
    for keep in faces:
        used[keep] = True
    key = v.copy()
    key[key == 0] = 0  # +0 and -0 compare equal
    rows = key.view(np.uint32)
    ids = np.nonzero(used)[0]
    _, first, inverse = np.unique(rows[ids], axis=0, return_index=True, return_inverse=True)
    rank = np.empty(len(first), np.int64)
    rank[np.argsort(first)] = np.arange(len(first))
    new_index = np.zeros(len(v), np.int64)
    new_index[ids] = rank[inverse.reshape(-1)]
    out_v = v[ids[np.sort(first)]]
    out_i = np.array([[new_index[k] for k in keep] if len(keep) == 3 else [0, 0, 0] for keep in faces],
                     np.uint32).reshape(-1)
    return out_v.astype(np.float32), out_i


def read_scn(path) -> tuple[dict, dict]:
    """A .scn file -> (raw scene dict, camera dict) (scenebuild.cpp:279-365)."""
    path = Path(path)
    text = path.read_text().replace("\r", "").replace("\t", "")
    lines = [l for l in text.split("\n") if l]
    cam = {"position": (F(0), F(0), F(0)), "lookdir": (F(0), F(0), F(-1)), "up": (F(0), F(1), F(0)),
           "fov_degrees": F(45), "near_plane": F(0.1), "far_plane": F(1000), "focus_dist": F(0),
           "lens_radius": F(0), "exposure": F(1)}
    env = (F(0), F(0), F(0))
    subs, order, have_camera = {}, [], False
    current, cur_tf = None, np.eye(4, dtype=np.float32)
    keys = {"fov": "fov_degrees", "near": "near_plane", "far": "far_plane", "focusdist": "focus_dist",
            "lensradius": "lens_radius", "exposure": "exposure"}
    i = 0
    section = None
    while i < len(lines):
        tk = _tokens(lines[i])
        i += 1
        if not tk:
            continue
        if tk[0].endswith(":"):
            if tk[0] not in ("camera:", "objects:"):
                raise ValueError("Unrecognised token " + tk[0])
            if tk[0] == "camera:":
                if have_camera:
                    raise ValueError("Camera already set.")
                have_camera = True
            if section == "objects:" and current is not None:
                subs[current][1].append(cur_tf)
                current = None
            section = tk[0]
            continue
        k = tk[0]
        if section == "camera:":
            if k in ("position", "lookdir", "up"):
                cam[k] = tuple(_stof(x) for x in tk[1:4])
            elif k in keys:
                cam[keys[k]] = _stof(tk[1])
            elif k == "envcol":
                env = tuple(from_srgb(_stof(x)) for x in tk[1:4])
            elif k == "envmap":
                pass
            else:
                raise ValueError("Unrecognised token in camera section " + k)
        elif section == "objects:":
            if k in ("t", "r", "s"):
                if current is None:
                    raise ValueError("no instance to transform")
                v = [_stof(x) for x in tk[1:]]
                M = _translation(*v) if k == "t" else _rotation(*v) if k == "r" else _scaling(*v)
                cur_tf = _mul(M, cur_tf)
            elif k in ("basecol", "roughness", "metalness", "specular"):
                pass
            elif k in ("plight", "dlight"):
                raise NotImplementedError("lights in .scn files")
            elif len(tk) == 1:
                if k not in subs:
                    raise ValueError(f"Object {k} not recognised.")
                if current is not None:
                    subs[current][1].append(cur_tf)
                current, cur_tf = k, np.eye(4, dtype=np.float32)
            else:
                subs[k] = (tk[1], [])
                order.append(k)
        else:
            raise ValueError("Unrecognised token " + k)
    if current is not None:
        subs[current][1].append(cur_tf)
    if not have_camera:
        raise ValueError("No camera section in scene description.")

    verts, idxs, meshes, mesh_mat, inst_off, insts, mats = [], [], [], [], [0], [], []
    vbase = ibase = mbase = 0
    for k in order:
        rel, scene_instances = subs[k]
        if not scene_instances:
            continue
        v, ix, ms, mm, mi, mt = read_gltf(path.parent / rel)
        if len(ms) != 1 or len(mt) != 1 or sum(len(x) for x in mi) != 1:
            raise NotImplementedError("the oracle's scene reader takes model files of one mesh, node and material")
        v, ix = assimp_single_mesh(v, ix)
        ms = [(0, 0, len(ix) // 3, len(v))]
        verts.append(v)
        idxs.append(ix)
        for m, (vo, io, tris, vc) in enumerate(ms):
            meshes.append((vo + vbase, io + ibase, tris, vc))
            mesh_mat.append(mm[m] + mbase)
            for si in scene_instances:
                for oi in mi[m]:
                    insts.append(_mul(si, oi).reshape(16))
            inst_off.append(len(insts))
        mats.append(mt)
        vbase += len(v)
        ibase += len(ix)
        mbase += len(mt)
    raw = {"vertices": np.concatenate(verts).astype(np.float32),
           "indices": np.concatenate(idxs).astype(np.uint32),
           "meshes": np.array(meshes, np.uint32).reshape(-1, 4),
           "mesh_material": np.array(mesh_mat, np.uint32),
           "mesh_instance_offset": np.array(inst_off, np.uint32),
           "instance_matrices": np.array(insts, np.float32).reshape(-1, 16),
           "materials": np.concatenate(mats).astype(np.float32),
           "point_lights": np.zeros((0, 6), np.float32), "directional_lights": np.zeros((0, 6), np.float32),
           "environment_colour": np.array(env, np.float32)}
    return raw, cam


def raw_struct(raw: dict):
    """raw dict -> pt_raw_scene (ctypes) + the arrays that must stay alive."""
    from pt_gb300 import abi  # struct layouts of include/pt_scene.h only
    keep = {k: np.ascontiguousarray(v) for k, v in raw.items() if isinstance(v, np.ndarray)}
    for k in ("point_lights", "directional_lights"):  # raw scenes of the generators may have none
        keep.setdefault(k, np.zeros((0, 6), np.float32))
    keep["environment_colour"] = np.asarray(raw.get("environment_colour", (0.0, 0.0, 0.0)), np.float32)

    def p(name, ct):
        return keep[name].ctypes.data_as(C.POINTER(ct))

    rs = abi.RawScene()
    rs.vertices = p("vertices", C.c_float)
    rs.vertex_count = keep["vertices"].size // 8
    rs.indices = p("indices", C.c_uint32)
    rs.index_count = keep["indices"].size
    rs.meshes = keep["meshes"].ctypes.data_as(C.POINTER(abi.MeshRange))
    rs.mesh_material = p("mesh_material", C.c_uint32)
    rs.mesh_instance_offset = p("mesh_instance_offset", C.c_uint32)
    rs.mesh_count = keep["mesh_material"].size
    rs.instance_matrices = p("instance_matrices", C.c_float)
    rs.instance_count = keep["instance_matrices"].size // 16
    rs.materials = keep["materials"].ctypes.data_as(C.POINTER(abi.Material))
    rs.material_count = keep["materials"].size // 24
    rs.point_lights = p("point_lights", C.c_float)
    rs.directional_lights = p("directional_lights", C.c_float)
    for k in range(3):
        rs.environment_colour[k] = float(keep["environment_colour"][k])
    return rs, keep


def camera_desc(cam: dict):
    from pt_gb300 import abi
    cd = abi.CameraDesc()
    for k in ("position", "lookdir", "up"):
        for i in range(3):
            getattr(cd, k)[i] = float(cam[k][i])
    for k in ("fov_degrees", "near_plane", "far_plane", "focus_dist", "lens_radius", "exposure"):
        setattr(cd, k, float(cam[k]))
    return cd
