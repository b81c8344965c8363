"""Seeded procedural scenes for the headless path, written in the reference's
drop-in formats: one `.scn` file (camera + objects + instances, README.md:25-52
of the reference) and one glTF 2.0 file (+ .bin) per object.

Random numbers come from the reference's host generator: xoshiro128++
(`Xshiro128`) seeded by four Splitmix32 outputs (src/rng.cpp), next_float =
next() / UINT32_MAX in float32.

Camera convention: the reference starts primary rays at -position and looks
along -lookdir (src/scene/camera.h:16 + src/pathtrace/pathtrace.cpp:387-388 +
src/scene/scenebuild.cpp:251-257), so a generator that wants the eye at E
looking at T writes `position -E` and `lookdir E - T`.

Scenes (configuration names follow the workload they model):
  small_scene  one 20x20 ground quad, 8 instances of a subdivision-3
               icosphere (1,280 tris) at xz ~ U[-4,4]^2 with scale U[0.5,1.5],
               albedo U[0.2,0.8]^3, a 2x2 emissive quad at y=6 (radiance 10),
               envcol 0.375 0.45 0.9, eye (-1,2,-3), fov 60, pinhole.
  mid_scene    ~260k instanced triangles from 200 instances of 6 meshes (two
               displaced 64x64 grids of 8,192 tris, two subdivision-4
               icospheres of 5,120 tris, two rounded boxes of 1,200 tris), four
               metallic-roughness materials per mesh (roughness U[0.05,1],
               metallic Bernoulli(0.3), base colour U[0.1,0.9]^3), 32 emissive
               triangles with strength log-uniform [1,100], thin lens
               (lensradius 0.03, focusdist 8).
"""
from __future__ import annotations

import json
import math
import struct
from pathlib import Path

import numpy as np

U32 = 0xFFFFFFFF


class SceneRng:
    """Xshiro128 (xoshiro128++) seeded with Splitmix32, as src/rng.cpp.

    Seeded the way the reference's only call site does it
    (lightsample.cpp:45-46, `Xshiro128 rng(seeder.next(), ... x4)`): with
    GCC's right-to-left evaluation of the arguments, the state holds the four
    Splitmix32 outputs in reverse order."""

    def __init__(self, seed: int):
        st = seed & U32
        s = []
        for _ in range(4):
            st = (st + 0x9E3779B9) & U32
            z = st
            z = ((z ^ (z >> 16)) * 0x85EBCA6B) & U32
            z = ((z ^ (z >> 13)) * 0xC2B2AE35) & U32
            s.append(z ^ (z >> 16))
        self.s = s[::-1]

    def next(self) -> int:
        s = self.s
        rotl = lambda x, k: ((x << k) | (x >> (32 - k))) & U32
        result = (rotl((s[0] + s[3]) & U32, 7) + s[0]) & U32
        t = (s[1] << 9) & U32
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = rotl(s[3], 11)
        return result

    def next_float(self) -> float:
        return float(np.float32(np.float32(self.next()) / np.float32(4294967295.0)))

    def uniform(self, lo: float, hi: float) -> float:
        return lo + (hi - lo) * self.next_float()


def to_srgb(x: float) -> float:
    return 12.92 * x if x <= 0.0031308 else 1.055 * x ** (1.0 / 2.4) - 0.055


# ---------------------------------------------------------------- meshes
# Each mesh: (positions (n,3), normals (n,3), uvs (n,2), indices (m,3)) float32/uint32.

def quad(size: float, y: float, facing_down: bool):
    h = size / 2
    p = np.array([[-h, y, -h], [h, y, -h], [h, y, h], [-h, y, h]], np.float32)
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    if facing_down:
        n = np.tile(np.array([[0, -1, 0]], np.float32), (4, 1))
        idx = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    else:
        n = np.tile(np.array([[0, 1, 0]], np.float32), (4, 1))
        idx = np.array([[0, 2, 1], [0, 3, 2]], np.uint32)
    return p, n, uv, idx


def icosphere(subdiv: int):
    t = (1.0 + 5 ** 0.5) / 2
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [tuple(c / math.sqrt(sum(x * x for x in v)) for c in v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache = {}
        new_faces = []

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                va, vb = verts[a], verts[b]
                m = [(va[k] + vb[k]) / 2 for k in range(3)]
                l = math.sqrt(sum(x * x for x in m))
                verts.append(tuple(x / l for x in m))
                cache[key] = len(verts) - 1
            return cache[key]

        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            new_faces += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = new_faces
    p = np.array(verts, np.float32)
    n = p.copy()
    u = 0.5 + np.arctan2(p[:, 2], p[:, 0]) / (2 * np.pi)
    v = np.arccos(np.clip(p[:, 1], -1, 1)) / np.pi
    uv = np.stack([u, v], 1).astype(np.float32)
    return p, n, uv, np.array(faces, np.uint32)


def displaced_grid(n: int, rng: SceneRng, amplitude: float = 0.08):
    waves = [(rng.uniform(1, 6), rng.uniform(1, 6), rng.uniform(0, 6.283), rng.uniform(0.3, 1.0)) for _ in range(4)]
    xs = np.linspace(-1, 1, n + 1, dtype=np.float64)
    X, Z = np.meshgrid(xs, xs, indexing="xy")

    def height(x, z):
        return amplitude * sum(a * np.sin(fx * x * 3.1416 + ph) * np.cos(fz * z * 3.1416 - ph) for fx, fz, ph, a in waves)

    Y = height(X, Z)
    e = 1e-4
    dx = (height(X + e, Z) - height(X - e, Z)) / (2 * e)
    dz = (height(X, Z + e) - height(X, Z - e)) / (2 * e)
    nrm = np.stack([-dx, np.ones_like(dx), -dz], -1)
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    p = np.stack([X, Y, Z], -1).reshape(-1, 3).astype(np.float32)
    uv = np.stack([(X + 1) / 2, (Z + 1) / 2], -1).reshape(-1, 2).astype(np.float32)
    return p, nrm.reshape(-1, 3).astype(np.float32), uv, grid_indices(n)


def grid_indices(n: int) -> np.ndarray:
    """Triangles of an (n+1)^2-vertex grid: per cell (row-major) (a, c, b), (b, c, d)."""
    j, i = np.meshgrid(np.arange(n, dtype=np.uint32), np.arange(n, dtype=np.uint32), indexing="ij")
    a = (j * (n + 1) + i).reshape(-1)
    b, c, d = a + 1, a + n + 1, a + n + 2
    return np.stack([np.stack([a, c, b], 1), np.stack([b, c, d], 1)], 1).reshape(-1, 3).astype(np.uint32)


def rounded_box(k: int, radius: float):
    """Cube with rounded edges from a k x k grid per face: 12 k^2 triangles."""
    pts, idx = [], []
    faces = [(0, 1, 2, 1), (0, 1, 2, -1), (1, 2, 0, 1), (1, 2, 0, -1), (2, 0, 1, 1), (2, 0, 1, -1)]
    for (ax, bx, nx, sgn) in faces:
        base = len(pts)
        for j in range(k + 1):
            for i in range(k + 1):
                c = [0.0, 0.0, 0.0]
                c[ax] = -1 + 2 * i / k
                c[bx] = -1 + 2 * j / k
                c[nx] = float(sgn)
                pts.append(c)
        for j in range(k):
            for i in range(k):
                a = base + j * (k + 1) + i
                b, cc, d = a + 1, a + k + 1, a + k + 2
                if sgn > 0:
                    idx += [(a, b, cc), (b, d, cc)]
                else:
                    idx += [(a, cc, b), (b, cc, d)]
    c = np.array(pts, np.float64)
    inner = np.clip(c, -(1 - radius), 1 - radius)
    d = c - inner
    dn = d / np.maximum(np.linalg.norm(d, axis=1, keepdims=True), 1e-12)
    p = inner + radius * dn
    uv = np.zeros((len(p), 2), np.float32)
    uv[:, 0] = (c[:, 0] + c[:, 2] + 2) / 4
    uv[:, 1] = (c[:, 1] + 1) / 2
    return p.astype(np.float32), dn.astype(np.float32), uv, np.array(idx, np.uint32)


def triangle(a, b, c):
    p = np.array([a, b, c], np.float32)
    nrm = np.cross(p[1] - p[0], p[2] - p[0])
    nrm = (nrm / np.linalg.norm(nrm)).astype(np.float32)
    return p, np.tile(nrm[None], (3, 1)), np.array([[0, 0], [1, 0], [0, 1]], np.float32), np.array([[0, 1, 2]], np.uint32)


# ---------------------------------------------------------------- writers

def write_gltf(path: Path, mesh, material: dict) -> None:
    """One mesh, one primitive, one node, one material; external .bin."""
    p, n, uv, idx = mesh
    p = np.ascontiguousarray(p, np.float32)
    n = np.ascontiguousarray(n, np.float32)
    uv = np.ascontiguousarray(uv, np.float32)
    idx = np.ascontiguousarray(idx, np.uint32).reshape(-1)
    blobs = [p.tobytes(), n.tobytes(), uv.tobytes(), idx.tobytes()]
    offsets, off = [], 0
    for b in blobs:
        offsets.append(off)
        off += (len(b) + 3) // 4 * 4
    binpath = path.with_suffix(".bin")
    with open(binpath, "wb") as f:
        for b in blobs:
            f.write(b)
            f.write(b"\0" * ((4 - len(b) % 4) % 4))
    views = [{"buffer": 0, "byteOffset": o, "byteLength": len(b)} for o, b in zip(offsets, blobs)]
    acc = [
        {"bufferView": 0, "componentType": 5126, "count": len(p), "type": "VEC3",
         "min": p.min(0).tolist(), "max": p.max(0).tolist()},
        {"bufferView": 1, "componentType": 5126, "count": len(n), "type": "VEC3"},
        {"bufferView": 2, "componentType": 5126, "count": len(uv), "type": "VEC2"},
        {"bufferView": 3, "componentType": 5125, "count": len(idx), "type": "SCALAR"},
    ]
    base = [float(to_srgb(c)) for c in material.get("base", (0.8, 0.8, 0.8))] + [1.0]
    mat = {"pbrMetallicRoughness": {"baseColorFactor": base, "metallicFactor": float(material.get("metallic", 0.0)),
                                    "roughnessFactor": float(material.get("roughness", 1.0))}}
    strength = float(material.get("emission_strength", 0.0))
    if strength > 0:
        mat["emissiveFactor"] = [1.0, 1.0, 1.0]
        mat["extensions"] = {"KHR_materials_emissive_strength": {"emissiveStrength": strength}}
    doc = {
        "asset": {"version": "2.0", "generator": "pt_gb300.scenes"},
        "scene": 0, "scenes": [{"nodes": [0]}], "nodes": [{"mesh": 0}],
        "meshes": [{"name": path.stem, "primitives": [{"attributes": {"POSITION": 0, "NORMAL": 1, "TEXCOORD_0": 2},
                                                        "indices": 3, "material": 0}]}],
        "materials": [mat],
        "accessors": acc, "bufferViews": views,
        "buffers": [{"uri": binpath.name, "byteLength": off}],
    }
    if strength > 0:
        doc["extensionsUsed"] = ["KHR_materials_emissive_strength"]
    path.write_text(json.dumps(doc))


def write_glb(path: Path, mesh, material: dict, base_colour_image: bytes | None = None,
              image_mime: str = "image/jpeg", lights: list | None = None) -> None:
    """One mesh as a binary glTF (.glb): the JSON chunk and one BIN chunk
    holding the vertex data and, optionally, an embedded base-colour image
    (PNG or JPEG bytes, referenced through a buffer view).  `lights`: a list
    of KHR_lights_punctual light dicts (type, color, intensity), each attached
    to a node of its own."""
    p, n, uv, idx = mesh
    blobs = [np.ascontiguousarray(p, np.float32).tobytes(), np.ascontiguousarray(n, np.float32).tobytes(),
             np.ascontiguousarray(uv, np.float32).tobytes(), np.ascontiguousarray(idx, np.uint32).reshape(-1).tobytes()]
    if base_colour_image is not None:
        blobs.append(bytes(base_colour_image))
    bin_chunk, offsets = bytearray(), []
    for b in blobs:
        offsets.append(len(bin_chunk))
        bin_chunk += b
        bin_chunk += b"\0" * ((4 - len(b) % 4) % 4)
    views = [{"buffer": 0, "byteOffset": o, "byteLength": len(b)} for o, b in zip(offsets, blobs)]
    acc = [
        {"bufferView": 0, "componentType": 5126, "count": len(p), "type": "VEC3",
         "min": np.asarray(p).min(0).tolist(), "max": np.asarray(p).max(0).tolist()},
        {"bufferView": 1, "componentType": 5126, "count": len(n), "type": "VEC3"},
        {"bufferView": 2, "componentType": 5126, "count": len(uv), "type": "VEC2"},
        {"bufferView": 3, "componentType": 5125, "count": int(np.asarray(idx).size), "type": "SCALAR"},
    ]
    pbr = {"metallicFactor": float(material.get("metallic", 0.0)), "roughnessFactor": float(material.get("roughness", 1.0))}
    doc = {"asset": {"version": "2.0", "generator": "pt_gb300.scenes"}, "scene": 0,
           "scenes": [{"nodes": [0]}], "nodes": [{"mesh": 0}],
           "meshes": [{"name": path.stem, "primitives": [{"attributes": {"POSITION": 0, "NORMAL": 1, "TEXCOORD_0": 2},
                                                          "indices": 3, "material": 0}]}],
           "materials": [{"pbrMetallicRoughness": pbr}], "accessors": acc, "bufferViews": views,
           "buffers": [{"byteLength": len(bin_chunk)}]}
    if base_colour_image is not None:
        doc["images"] = [{"bufferView": 4, "mimeType": image_mime}]
        doc["textures"] = [{"source": 0}]
        pbr["baseColorTexture"] = {"index": 0}
    else:
        pbr["baseColorFactor"] = [float(to_srgb(c)) for c in material.get("base", (0.8, 0.8, 0.8))] + [1.0]
    if lights:
        doc["extensionsUsed"] = ["KHR_lights_punctual"]
        doc["extensions"] = {"KHR_lights_punctual": {"lights": lights}}
        for i in range(len(lights)):
            doc["nodes"].append({"extensions": {"KHR_lights_punctual": {"light": i}}, "translation": [0.0, 3.0, 0.0]})
            doc["scenes"][0]["nodes"].append(len(doc["nodes"]) - 1)
    js = json.dumps(doc).encode()
    js += b" " * ((4 - len(js) % 4) % 4)
    body = struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(bin_chunk), 0x004E4942) + bytes(bin_chunk)
    path.write_bytes(struct.pack("<III", 0x46546C67, 2, 12 + len(body)) + body)


def fmt(x: float) -> str:
    return repr(float(np.float32(x)))


class ScnWriter:
    def __init__(self, camera: dict, env):
        self.camera = camera
        self.env = env
        self.objects = []   # (identifier, relative path)
        self.instances = []  # (identifier, [transform lines])

    def add_object(self, ident: str, rel: str):
        self.objects.append((ident, rel))

    def add_instance(self, ident: str, scale=None, rotate=None, translate=None):
        lines = []
        if scale is not None:
            lines.append("s " + " ".join(fmt(v) for v in scale))
        if rotate is not None:
            lines.append("r " + " ".join(fmt(v) for v in rotate))
        if translate is not None:
            lines.append("t " + " ".join(fmt(v) for v in translate))
        self.instances.append((ident, lines))

    def write(self, path: Path):
        eye, target = np.array(self.camera["eye"], np.float64), np.array(self.camera["target"], np.float64)
        out = ["camera:", "position " + " ".join(fmt(-v) for v in eye),
               "lookdir " + " ".join(fmt(v) for v in (eye - target)), "fov " + fmt(self.camera.get("fov", 45.0))]
        for key in ("near", "far", "focusdist", "lensradius", "exposure"):
            if key in self.camera:
                out.append(f"{key} {fmt(self.camera[key])}")
        out.append("envcol " + " ".join(fmt(v) for v in self.env))
        out.append("")
        out.append("objects:")
        for ident, rel in self.objects:
            out.append(f"{ident} {rel}")
        out.append("")
        for ident, lines in self.instances:
            out.append(ident)
            out += lines
            out.append("")
        path.write_text("\n".join(out) + "\n")


# ---------------------------------------------------------------- configurations

def small_scene(out_dir: Path, seed: int = 0) -> Path:
    out_dir = Path(out_dir)
    out_dir.mkdir(parents=True, exist_ok=True)
    rng = SceneRng(seed)
    albedo = lambda: tuple(rng.uniform(0.2, 0.8) for _ in range(3))
    write_gltf(out_dir / "ground.gltf", quad(20.0, 0.0, False), {"base": albedo(), "roughness": 1.0, "metallic": 0.0})
    write_gltf(out_dir / "sphere.gltf", icosphere(3), {"base": albedo(), "roughness": 1.0, "metallic": 0.0})
    write_gltf(out_dir / "light.gltf", quad(2.0, 6.0, True),
               {"base": (0.0, 0.0, 0.0), "roughness": 1.0, "metallic": 0.0, "emission_strength": 10.0})
    scn = ScnWriter({"eye": (-1.0, 2.0, -3.0), "target": (0.0, 0.75, 0.0), "fov": 60.0}, (0.375, 0.45, 0.9))
    for name in ("ground", "sphere", "light"):
        scn.add_object(name, f"{name}.gltf")
    scn.add_instance("ground")
    for _ in range(8):
        x, z, s = rng.uniform(-4, 4), rng.uniform(-4, 4), rng.uniform(0.5, 1.5)
        scn.add_instance("sphere", scale=(s, s, s), translate=(x, s, z))
    scn.add_instance("light")
    path = out_dir / "small.scn"
    scn.write(path)
    return path


def mid_scene(out_dir: Path, seed: int = 1) -> Path:
    out_dir = Path(out_dir)
    out_dir.mkdir(parents=True, exist_ok=True)
    rng = SceneRng(seed)
    meshes = {
        "grid0": displaced_grid(64, rng), "grid1": displaced_grid(64, rng),
        "sphere0": icosphere(4), "sphere1": icosphere(4),
        "box0": rounded_box(10, 0.15), "box1": rounded_box(10, 0.3),
    }
    palettes = {}
    scn = ScnWriter({"eye": (0.0, 5.0, -22.0), "target": (0.0, 1.0, 0.0), "fov": 45.0, "focusdist": 8.0,
                     "lensradius": 0.03}, (0.2, 0.25, 0.4))
    for name, mesh in meshes.items():
        palettes[name] = []
        for k in range(4):
            mat = {"base": tuple(rng.uniform(0.1, 0.9) for _ in range(3)), "roughness": rng.uniform(0.05, 1.0),
                   "metallic": 1.0 if rng.next_float() < 0.3 else 0.0}
            ident = f"{name}_m{k}"
            write_gltf(out_dir / f"{ident}.gltf", mesh, mat)
            palettes[name].append(ident)
    used = set()
    instances = []
    # terrain tiles
    for i, name in enumerate(("grid0", "grid1")):
        instances.append((palettes[name][rng.next() % 4], (10.0, 10.0, 10.0), None, (-10.0 + 20.0 * i, 0.0, 0.0)))
    for name in ("sphere0", "sphere1"):
        s = rng.uniform(1.5, 3.0)
        instances.append((palettes[name][rng.next() % 4], (s, s, s), None, (rng.uniform(-12, 12), s, rng.uniform(-4, 8))))
    for i in range(196):
        name = "box0" if i % 2 == 0 else "box1"
        s = rng.uniform(0.3, 1.0)
        axis = (rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(-1, 1))
        angle = rng.uniform(1e-5, 2 * math.pi)
        pos = (rng.uniform(-18, 18), s + rng.uniform(0.0, 1.5), rng.uniform(-8, 9))
        instances.append((palettes[name][rng.next() % 4], (s, s, s), axis + (angle,), pos))
    for ident, s, r, t in instances:
        used.add(ident)
    for name, idents in palettes.items():
        for ident in idents:
            if ident in used:
                scn.add_object(ident, f"{ident}.gltf")
    for ident, s, r, t in instances:
        scn.add_instance(ident, scale=s, rotate=r, translate=t)
    for e in range(32):
        cx, cy, cz = rng.uniform(-16, 16), rng.uniform(6, 10), rng.uniform(-6, 10)
        size = rng.uniform(0.6, 1.4)
        a = (cx - size, cy, cz - size * 0.5)
        b = (cx + size, cy, cz - size * 0.5)
        c = (cx, cy, cz + size)
        strength = math.exp(rng.uniform(math.log(1.0), math.log(100.0)))
        ident = f"emitter{e}"
        write_gltf(out_dir / f"{ident}.gltf", triangle(a, c, b),
                   {"base": (0.0, 0.0, 0.0), "roughness": 1.0, "metallic": 0.0, "emission_strength": strength})
        scn.add_object(ident, f"{ident}.gltf")
        scn.add_instance(ident)
    path = out_dir / "mid.scn"
    scn.write(path)
    return path


def tiny_raw(kind: str = "two_tris") -> tuple[dict, dict]:
    """Very small raw scenes for exhaustive parity tests (no files)."""
    mats = []

    def material(base, rough=0.5, metal=0.0, emission=0.0, alpha=1.0):
        m = np.zeros(24, np.float32)
        m[0:3] = base
        m[3] = alpha
        m[4:7] = 1.0 if emission > 0 else 0.0
        m[7] = emission if emission > 0 else 1.0
        m[8] = rough
        m[9] = metal
        bits = (1 << 13) if alpha < 1.0 else 0
        m[11] = np.frombuffer(np.uint32(bits).tobytes(), np.float32)[0]
        m[12:15] = 0.5
        m[21] = 0.5
        mats.append(m)
        return len(mats) - 1

    meshes = []
    if kind == "two_tris":
        meshes.append((quad(4.0, 0.0, False), material((0.7, 0.6, 0.5), 0.6, 0.0), [np.eye(4, dtype=np.float32)]))
        meshes.append((quad(1.0, 2.0, True), material((0.0, 0.0, 0.0), emission=5.0), [np.eye(4, dtype=np.float32)]))
    else:
        raise ValueError(kind)
    v, idx, ranges, mm, mio, inst = [], [], [], [], [0], []
    voff = ioff = 0
    for (p, n, uv, ix), mat, insts in meshes:
        v.append(np.concatenate([p, n, uv], 1))
        idx.append(ix.reshape(-1))
        ranges.append((voff, ioff, len(ix), len(p)))
        voff += len(p)
        ioff += ix.size
        mm.append(mat)
        for M in insts:
            inst.append(np.asarray(M, np.float32).T.reshape(-1))  # column-major
        mio.append(mio[-1] + len(insts))
    raw = {"vertices": np.concatenate(v).astype(np.float32), "indices": np.concatenate(idx).astype(np.uint32),
           "meshes": np.array(ranges, np.uint32), "mesh_material": np.array(mm, np.uint32),
           "mesh_instance_offset": np.array(mio, np.uint32), "instance_matrices": np.array(inst, np.float32),
           "materials": np.array(mats, np.float32), "environment_colour": np.array([0.1, 0.15, 0.3], np.float32)}
    # eye (0, 1.5, 4) looking at the origin: position -eye, lookdir eye - target
    cam = {"position": (0.0, -1.5, -4.0), "lookdir": (0.0, 1.5, 4.0), "fov_degrees": 50.0}
    return raw, cam


def material_row(base, rough=0.5, metal=0.0, emission=0.0, alpha=1.0) -> np.ndarray:
    """One pt_material row (24 floats).  alpha < 1 sets the transparency bit,
    as the scene builder does for KHR_materials_transmission (opacity =
    1 - transmission, scene.cpp:96-108)."""
    m = np.zeros(24, np.float32)
    m[0:3] = base
    m[3] = alpha
    m[4:7] = 1.0 if emission > 0 else 0.0
    m[7] = emission if emission > 0 else 1.0
    m[8] = rough
    m[9] = metal
    bits = (1 << 13) if alpha < 1.0 else 0
    m[11] = np.frombuffer(np.uint32(bits).tobytes(), np.float32)[0]
    m[12:15] = 0.5
    m[21] = 0.5
    return m


def assemble_raw(meshes, env) -> dict:
    """meshes: [((p, n, uv, ix), material row, [4x4 object-to-world matrices])]."""
    v, idx, ranges, mm, mio, inst, mats = [], [], [], [], [0], [], []
    voff = ioff = 0
    for (p, n, uv, ix), mat, insts in meshes:
        v.append(np.concatenate([p, n, uv], 1))
        idx.append(ix.reshape(-1))
        ranges.append((voff, ioff, len(ix), len(p)))
        voff += len(p)
        ioff += ix.size
        mats.append(mat)
        mm.append(len(mats) - 1)
        for M in insts:
            inst.append(np.asarray(M, np.float32).T.reshape(-1))  # column-major
        mio.append(mio[-1] + len(insts))
    return {"vertices": np.concatenate(v).astype(np.float32), "indices": np.concatenate(idx).astype(np.uint32),
            "meshes": np.array(ranges, np.uint32), "mesh_material": np.array(mm, np.uint32),
            "mesh_instance_offset": np.array(mio, np.uint32), "instance_matrices": np.array(inst, np.float32),
            "materials": np.array(mats, np.float32), "environment_colour": np.asarray(env, np.float32)}


def glass_raw(kind: str = "glass") -> tuple[dict, dict]:
    """Scenes for the refractive dielectric (raw["material_ior"], an extension
    of this library).  "glass": a diffuse ground lit by an emissive quad, a
    clear glass icosphere (index 1.5), a green-tinted one (1.33) and a rough
    metal one.  "furnace": one clear glass icosphere (index 1.5) alone in a
    uniform white environment and no lights; a lossless dielectric keeps every
    pixel at radiance 1 when Russian roulette is off (the white furnace test)."""
    p, n, uv, ix = icosphere(3)
    if kind == "furnace":
        raw = assemble_raw([((p, n, uv, ix), material_row((1.0, 1.0, 1.0), 0.5), [np.eye(4)])], (1.0, 1.0, 1.0))
        raw["material_ior"] = np.array([1.5], np.float32)
        cam = {"position": (0.0, 0.0, -3.0), "lookdir": (0.0, 0.0, 3.0), "fov_degrees": 45.0}
        return raw, cam
    if kind != "glass":
        raise ValueError(kind)

    def at(x, y, z, s):
        M = np.eye(4)
        M[:3, :3] *= s
        M[:3, 3] = (x, y, z)
        return M

    meshes = [(quad(6.0, 0.0, False), material_row((0.7, 0.65, 0.55), 0.8), [np.eye(4)]),
              (quad(1.2, 3.0, True), material_row((0, 0, 0), 1.0, 0.0, 12.0), [np.eye(4)]),
              ((p, n, uv, ix), material_row((1.0, 1.0, 1.0), 0.5), [at(-1.1, 0.7, 0.0, 0.7)]),
              ((p, n, uv, ix), material_row((0.6, 0.95, 0.7), 0.5), [at(0.5, 0.5, 0.6, 0.5)]),
              ((p, n, uv, ix), material_row((0.9, 0.8, 0.6), 0.3, 1.0), [at(1.2, 0.6, -0.8, 0.6)])]
    raw = assemble_raw(meshes, (0.1, 0.15, 0.3))
    raw["material_ior"] = np.array([0.0, 0.0, 1.5, 1.33, 0.0], np.float32)
    cam = {"position": (0.0, -1.8, -4.5), "lookdir": (0.0, 1.3, 4.5), "fov_degrees": 50.0}
    return raw, cam


def _bits(i: int) -> np.float32:
    return np.frombuffer(np.uint32(i).tobytes(), np.float32)[0]


def textured_raw(seed: int = 4) -> tuple[dict, dict]:
    """A small raw scene that reads every texture path of the shader:
    a ground quad with an sRGB base-colour map whose alpha dips below one
    (transparency), a combined roughness-metalness map and a normal map, with
    texture coordinates running over [-0.7, 1.8) so that REPEAT wraps them;
    an icosphere with 1-channel roughness, 2-channel metalness, specular and
    sheen maps; a box with a plain material; an emissive quad whose emission
    map makes it a textured emitter (light intensity by the reference's
    20-sample estimate, light samples reading the map at their uv)."""
    rng = np.random.default_rng(seed)
    tex = []

    def add(img, srgb):
        tex.append((np.ascontiguousarray(img, np.uint8), srgb))
        return len(tex) - 1

    h, w = 48, 64
    yy, xx = np.mgrid[0:h, 0:w]
    check = ((xx // 8 + yy // 8) % 2).astype(np.float32)
    base = np.zeros((h, w, 4), np.uint8)
    base[..., 0] = 40 + 180 * check
    base[..., 1] = 60 + 150 * (xx / (w - 1))
    base[..., 2] = 200 - 150 * (yy / (h - 1))
    base[..., 3] = np.where((xx // 16 + yy // 16) % 3 == 0, 96, 255)
    t_base = add(base, True)
    mr = rng.integers(0, 256, (32, 32, 4), dtype=np.uint8)
    mr[..., 2] = np.where(mr[..., 2] > 200, 255, 0)
    t_mr = add(mr, False)
    nx = 0.35 * np.sin(np.mgrid[0:32, 0:32][1] * 0.6)
    ny = 0.35 * np.cos(np.mgrid[0:32, 0:32][0] * 0.45)
    nz = np.sqrt(1 - nx * nx - ny * ny)
    nrm = np.stack([nx, ny, nz, np.ones_like(nx)], -1)
    t_normal = add(np.round((nrm * 0.5 + 0.5) * 255), False)
    t_rough = add(rng.integers(20, 256, (16, 24), dtype=np.uint8), False)
    t_metal = add(rng.integers(0, 256, (8, 8, 2), dtype=np.uint8), False)
    t_spec = add(rng.integers(0, 256, (8, 12, 4), dtype=np.uint8), False)
    t_sheen = add(rng.integers(0, 128, (4, 4, 4), dtype=np.uint8), False)
    em = np.zeros((16, 16, 4), np.uint8)
    em[..., 0] = 255
    em[..., 1] = np.linspace(40, 255, 16)[None, :]
    em[..., 2] = np.linspace(255, 20, 16)[:, None]
    em[..., 3] = 255
    t_emit = add(em, True)

    def mat(**kw):
        m = material_row(kw.get("base", (0.8, 0.8, 0.8)), kw.get("rough", 0.5), kw.get("metal", 0.0),
                         kw.get("emission", 0.0))
        bits = 0
        for key, bit, slot in (("base_map", 1 << 0, 0), ("emission_map", 1 << 1, 4), ("rough_map", 1 << 2, 8),
                               ("metal_map", 1 << 3, 9), ("rm_map", 1 << 4, 8), ("spec_map", 1 << 5, 12),
                               ("sheen_map", 1 << 7, 16), ("normal_map", 1 << 12, 10)):
            if key in kw:
                bits |= bit
                m[slot] = _bits(kw[key])
        if kw.get("transparent"):
            bits |= 1 << 13
        m[11] = _bits(bits)
        return m

    p, n, uv, ix = quad(6.0, 0.0, False)
    ground = (p, n, (uv * 2.5 - 0.7).astype(np.float32), ix)
    sp, sn, suv, six = icosphere(2)
    boxp, boxn, boxuv, boxix = rounded_box(2, 0.1)
    lp, ln_, luv, lix = quad(1.5, 3.0, True)
    eye = np.eye(4, dtype=np.float32)
    sphere_m = np.diag([0.8, 0.8, 0.8, 1]).astype(np.float32)
    sphere_m[:3, 3] = (-0.9, 0.8, 0.2)
    box_m = np.diag([0.6, 0.9, 0.6, 1]).astype(np.float32)
    box_m[:3, 3] = (1.1, 0.9, -0.6)
    raw = assemble_raw([
        (ground, mat(base_map=t_base, rm_map=t_mr, normal_map=t_normal, transparent=True), [eye]),
        ((sp, sn, suv, six), mat(base=(0.9, 0.5, 0.3), rough_map=t_rough, metal_map=t_metal, spec_map=t_spec,
                                 sheen_map=t_sheen), [sphere_m]),
        ((boxp, boxn, boxuv, boxix), mat(base=(0.3, 0.7, 0.4), rough=0.3), [box_m]),
        ((lp, ln_, luv, lix), mat(base=(0, 0, 0), emission=6.0, emission_map=t_emit), [eye]),
    ], (0.05, 0.07, 0.12))
    raw["point_lights"] = np.array([[2.5, 2.0, 2.5, 3.0, 2.5, 2.0]], np.float32)
    raw["textures"] = tex
    # eye (0.5, 3.2, 4.5) looking at (0, 0.4, 0)
    cam = {"position": (-0.5, -3.2, -4.5), "lookdir": (0.5, 2.8, 4.5), "fov_degrees": 55.0}
    return raw, cam


_ICOSPHERES: dict = {}


def _icosphere_cached(subdiv: int):
    if subdiv not in _ICOSPHERES:
        _ICOSPHERES[subdiv] = icosphere(subdiv)
    return _ICOSPHERES[subdiv]


def batch_scene(seed: int, tris: int) -> tuple[dict, dict]:
    """One job scene of the batch workload with about `tris` unique triangles:
    a 12x12 ground quad, a displaced grid holding ~70 % of the triangles
    (scaled 3x, at the centre), an icosphere of subdivision s (20 * 4^s
    triangles, ~30 %) instanced 3-8 times, 1-3 emissive quads (strength
    log-uniform [2, 40]), roughness U[0.05, 1], metallic Bernoulli(0.3), base
    colour U[0.1, 0.9]^3, eye on a circle of radius U[5, 9] at height
    U[1.5, 4] looking at the origin, fov U[35, 65]."""
    rng = np.random.default_rng(seed)
    srng = SceneRng(seed)

    def mat(**kw):
        return material_row(rng.uniform(0.1, 0.9, 3), float(rng.uniform(0.05, 1.0)), float(rng.random() < 0.3), **kw)

    n = max(2, int(round(math.sqrt(0.35 * tris))))
    sub = int(min(6, max(0, round(math.log(max(0.3 * tris, 20) / 20, 4)))))
    grid = displaced_grid(n, srng, amplitude=0.12)
    gm = np.diag([3.0, 3.0, 3.0, 1.0]).astype(np.float32)
    meshes = [(quad(12.0, -0.4, False), mat(), [np.eye(4, dtype=np.float32)]),
              (grid, mat(), [gm])]
    sphere_insts = []
    for _ in range(int(rng.integers(3, 9))):
        m = np.diag([rng.uniform(0.3, 0.8)] * 3 + [1.0]).astype(np.float32)
        m[:3, 3] = (rng.uniform(-4, 4), rng.uniform(0.2, 1.5), rng.uniform(-4, 4))
        sphere_insts.append(m)
    meshes.append((_icosphere_cached(sub), mat(), sphere_insts))
    for _ in range(int(rng.integers(1, 4))):
        m = np.eye(4, dtype=np.float32)
        m[:3, 3] = (rng.uniform(-3, 3), rng.uniform(3.5, 5.5), rng.uniform(-3, 3))
        meshes.append((quad(float(rng.uniform(0.8, 2.0)), 0.0, True),
                       material_row((0, 0, 0), emission=float(math.exp(rng.uniform(math.log(2), math.log(40))))), [m]))
    raw = assemble_raw(meshes, rng.uniform(0.05, 0.4, 3).astype(np.float32))
    ang = rng.uniform(0, 2 * math.pi)
    r = rng.uniform(5, 9)
    eye = np.array([r * math.cos(ang), rng.uniform(1.5, 4.0), r * math.sin(ang)], np.float32)
    cam = {"position": tuple(-eye), "lookdir": tuple(eye), "fov_degrees": float(rng.uniform(35, 65))}
    return raw, cam


def batch_workload(seed: int = 7, jobs: int = 64, side=(128, 1024), spp=(4, 256), tris=(1000, 500000),
                   max_bounces: int = 8) -> list[dict]:
    """The batch workload: `jobs` render jobs with image side log-uniform in
    `side` (square images, side rounded to a multiple of 8), samples
    log-uniform in `spp` (integer) and unique triangles log-uniform in `tris`,
    each with its own scene (batch_scene).  Returns dicts with keys seed,
    side, spp, tris, max_bounces."""
    rng = np.random.default_rng(seed)

    def logu(lo, hi):
        return math.exp(rng.uniform(math.log(lo), math.log(hi)))

    out = []
    for j in range(jobs):
        out.append({"seed": seed * 1000 + j, "side": int(round(logu(*side) / 8)) * 8, "spp": int(round(logu(*spp))),
                    "tris": int(round(logu(*tris))), "max_bounces": max_bounces})
    return out


def png_bytes(img: np.ndarray) -> bytes:
    """Encode an 8-bit image ([h, w] or [h, w, c], c in 1..4) as PNG
    (filter 0 rows, one zlib stream)."""
    import zlib
    img = np.ascontiguousarray(img, np.uint8)
    h, w = img.shape[:2]
    c = 1 if img.ndim == 2 else img.shape[2]
    ctype = {1: 0, 2: 4, 3: 2, 4: 6}[c]
    rows = b"".join(b"\0" + img[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & U32)

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(rows)) + chunk(b"IEND", b""))


def _displaced_sphere(subdiv: int, rng: np.random.Generator):
    p, n, uv, ix = icosphere(subdiv)
    waves = rng.uniform(1, 5, (3, 3))
    ph = rng.uniform(0, 6.283, 3)
    d = 1.0 + 0.06 * sum(np.sin(p @ waves[k] * 3.0 + ph[k]) for k in range(3))
    return (p * d[:, None]).astype(np.float32), n, uv, ix


def heavy_scene(seed: int = 3, instances: int = 10000, grids: int = 32, spheres: int = 32, grid_n: int = 144,
                sphere_subdiv: int = 5, emitters: int = 256, dielectric: bool = False):
    """The heavy benchmark scene as a raw scene: 64 BLASes totalling ~2M unique
    triangles (32 displaced 144x144 grids of 41,472 triangles, 32 displaced
    subdivision-5 icospheres of 20,480), 10,000 instances with random rotation
    (angle U(1e-5, 2 pi)), scale and translation, 10 % of the meshes
    transmissive (opacity 0.1: the reference maps glTF transmission to
    opacity), 256 single-triangle emitters with radiance log-uniform in
    [1, 100].  Returns (raw, camera) for HostScene.from_raw; render at
    1920x1080 with 12 bounces and Russian roulette from segment 4.  With
    `dielectric` the transmissive meshes are opaque refractive dielectrics of
    index 1.5 instead (raw["material_ior"]; the same random draws otherwise)."""
    rng = np.random.default_rng(seed)
    srng = SceneRng(seed)
    base = [displaced_grid(grid_n, srng, amplitude=0.1) for _ in range(grids)] + \
           [_displaced_sphere(sphere_subdiv, rng) for _ in range(spheres)]
    mats, glass = [], []
    for k in range(len(base)):
        transmissive = rng.random() < 0.1
        mats.append(material_row(rng.uniform(0.1, 0.9, 3), rng.uniform(0.05, 1.0),
                                 1.0 if rng.random() < 0.3 else 0.0,
                                 alpha=0.1 if transmissive and not dielectric else 1.0))
        glass.append(transmissive and dielectric)
    per_mesh = [[] for _ in base]
    for i in range(instances):
        k = int(rng.integers(len(base)))
        axis = rng.uniform(-1, 1, 3)
        axis /= max(np.linalg.norm(axis), 1e-9)
        ang = rng.uniform(1e-5, 2 * math.pi)
        x, y, z = axis
        c, s_, C = math.cos(ang), math.sin(ang), 1 - math.cos(ang)
        R = np.array([[c + x * x * C, x * y * C - z * s_, x * z * C + y * s_],
                      [y * x * C + z * s_, c + y * y * C, y * z * C - x * s_],
                      [z * x * C - y * s_, z * y * C + x * s_, c + z * z * C]])
        sc = rng.uniform(0.3, 2.5)
        M = np.eye(4)
        M[:3, :3] = R * sc
        M[:3, 3] = (rng.uniform(-120, 120), rng.uniform(0, 25), rng.uniform(-120, 120))
        per_mesh[k].append(M)
    meshes = [(m, mat, ms) for m, mat, ms in zip(base, mats, per_mesh) if ms]
    ior = [1.5 if g else 0.0 for g, ms in zip(glass, per_mesh) if ms]
    for e in range(emitters):
        cx, cy, cz = rng.uniform(-110, 110), rng.uniform(30, 45), rng.uniform(-110, 110)
        size = rng.uniform(1.0, 4.0)
        tri = triangle((cx - size, cy, cz - size * 0.5), (cx, cy, cz + size), (cx + size, cy, cz - size * 0.5))
        strength = float(math.exp(rng.uniform(0.0, math.log(100.0))))
        meshes.append((tri, material_row((0, 0, 0), 1.0, 0.0, strength), [np.eye(4)]))
    raw = assemble_raw(meshes, (0.25, 0.3, 0.45))
    if dielectric:
        raw["material_ior"] = np.array(ior + [0.0] * emitters, np.float32)
    eye, target = np.array([0.0, 60.0, -170.0]), np.array([0.0, 5.0, 0.0])
    cam = {"position": tuple(-eye), "lookdir": tuple(eye - target), "fov_degrees": 50.0}
    return raw, cam
