"""Seeded procedural scenes for training the denoiser.

Each scene mixes the building blocks of the benchmark scenes (displaced
grids, icospheres, beveled boxes, single-triangle emitters with radiance
log-uniform in [1, 100], metallic-roughness materials with roughness
U[0.05, 1], metallic Bernoulli(0.3), base colour U[0.1, 0.9]^3) with random
counts, scales, sky colour and cameras (field of view log-uniform in [8, 60]
degrees, so that 256-pixel frames span the pixel footprints of 256^2 to
1920-wide renders; thin lens), and goes straight to the library as a raw
scene (no files).
"""
from __future__ import annotations

import math

import numpy as np

from . import scenes


def material(base, rough=0.5, metal=0.0, emission=0.0, alpha=1.0) -> np.ndarray:
    """One pt_material row (24 floats, include/pt_gpu.h layout); alpha < 1
    sets the transparency bit (transmission as the reference maps it)."""
    m = np.zeros(24, np.float32)
    m[0:3] = base
    m[3] = alpha
    if alpha < 1.0:
        m[11] = np.frombuffer(np.uint32(1 << 13).tobytes(), np.float32)[0]
    m[4:7] = 1.0 if emission > 0 else 0.0
    m[7] = emission if emission > 0 else 1.0
    m[8] = rough
    m[9] = metal
    m[12:15] = 0.5
    m[21] = 0.5
    return m


def _rotation(axis, angle) -> np.ndarray:
    a = np.asarray(axis, np.float64)
    a = a / max(np.linalg.norm(a), 1e-9)
    x, y, z = a
    c, s = math.cos(angle), math.sin(angle)
    C = 1 - c
    return np.array([[c + x * x * C, x * y * C - z * s, x * z * C + y * s],
                     [y * x * C + z * s, c + y * y * C, y * z * C - x * s],
                     [z * x * C - y * s, z * y * C + x * s, c + z * z * C]])


def _matrix(scale, rot, pos) -> np.ndarray:
    M = np.eye(4)
    M[:3, :3] = rot @ np.diag(scale)
    M[:3, 3] = pos
    return M


_LIB: dict | None = None


def _mesh_library():
    global _LIB
    if _LIB is None:
        rng = scenes.SceneRng(12345)
        _LIB = {"grid": [scenes.displaced_grid(48, rng), scenes.displaced_grid(48, rng, amplitude=0.15)],
                "sphere": [scenes.icosphere(3), scenes.icosphere(4)],
                "box": [scenes.rounded_box(8, 0.15), scenes.rounded_box(8, 0.3)],
                "ground": [scenes.quad(1.0, 0.0, False)]}
    return _LIB


def render_settings(seed: int) -> tuple[int, int]:
    """(max bounces, first Russian-roulette segment) of training scene `seed`:
    the benchmark's 8 / 1 for 70 % of the scenes, 12 / 4 (the heavy
    configuration's) for the rest."""
    rng = np.random.default_rng([seed, 7])
    return (8, 1) if rng.random() < 0.7 else (12, 4)


def training_scene(seed: int):
    """Returns (raw scene dict, camera dict) for HostScene.from_raw.  A quarter
    of the scenes are "clutter" scenes modelled on the heavy configuration
    (hundreds to thousands of randomly rotated instances of displaced grids
    and spheres in a wide volume, 10 % of the variants transmissive, emitters
    above, a distant camera); the rest are ground + objects scenes."""
    rng = np.random.default_rng(seed)
    if rng.random() < 0.25:
        return _clutter_scene(rng)
    lib = _mesh_library()
    meshes = []  # (mesh arrays, material row, [4x4 matrices])

    def rand_material():
        return material(rng.uniform(0.1, 0.9, 3), rng.uniform(0.05, 1.0), 1.0 if rng.random() < 0.3 else 0.0)

    # ground: a flat quad or displaced tiles
    if rng.random() < 0.5:
        s = rng.uniform(20, 40)
        meshes.append((lib["ground"][0], rand_material(), [_matrix((s, 1, s), np.eye(3), (0, 0, 0))]))
    else:
        g = lib["grid"][rng.integers(2)]
        mats = []
        for i in range(2):
            mats.append(_matrix((10, 10, 10), np.eye(3), (-10 + 20 * i, 0, 0)))
        meshes.append((g, rand_material(), mats))
    # objects in a few material variants per mesh kind
    n_boxes = int(rng.integers(0, 160))
    n_spheres = int(rng.integers(0, 8))
    for kind, count in (("box", n_boxes), ("sphere", n_spheres)):
        if count == 0:
            continue
        variants = [(lib[kind][rng.integers(2)], rand_material(), []) for _ in range(4)]
        for i in range(count):
            if kind == "box":
                s = rng.uniform(0.3, 1.0)
                rot = _rotation(rng.uniform(-1, 1, 3), rng.uniform(1e-5, 2 * math.pi))
                pos = (rng.uniform(-18, 18), s + rng.uniform(0, 1.5), rng.uniform(-8, 9))
            else:
                s = rng.uniform(0.8, 3.0)
                rot = np.eye(3)
                pos = (rng.uniform(-12, 12), s, rng.uniform(-4, 8))
            variants[rng.integers(4)][2].append(_matrix((s, s, s), rot, pos))
        meshes += [v for v in variants if v[2]]
    # emitters: single triangles, radiance log-uniform [1, 100]
    n_em = int(np.exp(rng.uniform(0, math.log(32))))
    for _ in range(n_em):
        cx, cy, cz = rng.uniform(-16, 16), rng.uniform(4, 10), rng.uniform(-6, 10)
        size = rng.uniform(0.5, 1.5)
        tri = scenes.triangle((cx - size, cy, cz - size * 0.5), (cx, cy, cz + size), (cx + size, cy, cz - size * 0.5))
        strength = float(np.exp(rng.uniform(0, math.log(100))))
        meshes.append((tri, material((0, 0, 0), 1.0, 0.0, strength), [np.eye(4)]))

    return _assemble(meshes, rng), _camera(rng)


def _clutter_scene(rng):
    lib = _mesh_library()
    kinds = lib["grid"] + lib["sphere"]
    variants = []
    for _ in range(int(rng.integers(4, 12))):
        alpha = float(rng.uniform(0.1, 0.5)) if rng.random() < 0.1 else 1.0
        m = material(rng.uniform(0.1, 0.9, 3), rng.uniform(0.05, 1.0), 1.0 if rng.random() < 0.3 else 0.0, alpha=alpha)
        variants.append((kinds[rng.integers(len(kinds))], m, []))
    extent = float(rng.uniform(20, 120))
    for _ in range(int(np.exp(rng.uniform(math.log(200), math.log(3000))))):
        s = rng.uniform(0.3, 2.5)
        rot = _rotation(rng.uniform(-1, 1, 3), rng.uniform(1e-5, 2 * math.pi))
        pos = (rng.uniform(-extent, extent), rng.uniform(0, 0.2 * extent), rng.uniform(-extent, extent))
        variants[rng.integers(len(variants))][2].append(_matrix((s, s, s), rot, pos))
    meshes = [v for v in variants if v[2]]
    for _ in range(int(np.exp(rng.uniform(math.log(8), math.log(256))))):
        cx, cy, cz = rng.uniform(-extent, extent), rng.uniform(0.25, 0.4) * extent, rng.uniform(-extent, extent)
        size = rng.uniform(0.01, 0.035) * extent
        tri = scenes.triangle((cx - size, cy, cz - size * 0.5), (cx, cy, cz + size), (cx + size, cy, cz - size * 0.5))
        strength = float(np.exp(rng.uniform(0, math.log(100))))
        meshes.append((tri, material((0, 0, 0), 1.0, 0.0, strength), [np.eye(4)]))
    raw = _assemble(meshes, rng)
    eye = np.array([rng.uniform(-0.3, 0.3) * extent, rng.uniform(0.2, 0.6) * extent, -rng.uniform(0.9, 1.6) * extent])
    target = np.array([rng.uniform(-0.2, 0.2) * extent, rng.uniform(0.0, 0.1) * extent, rng.uniform(-0.2, 0.2) * extent])
    fov = float(np.exp(rng.uniform(math.log(20), math.log(60))))
    cam = {"position": tuple(-eye), "lookdir": tuple(eye - target), "fov_degrees": fov}
    return raw, cam


def _assemble(meshes, rng) -> dict:
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
    env = rng.uniform(0.05, 0.5, 3) * np.array([0.7, 0.8, 1.0])
    return {"vertices": np.concatenate(v).astype(np.float32), "indices": np.concatenate(idx).astype(np.uint32),
            "meshes": np.array(ranges, np.uint32), "mesh_material": np.array(mm, np.uint32),
            "mesh_instance_offset": np.array(mio, np.uint32), "instance_matrices": np.array(inst, np.float32),
            "materials": np.array(mats, np.float32), "environment_colour": env.astype(np.float32)}


def _camera(rng) -> dict:
    # camera: eye around the scene looking at a point near the centre
    dist = rng.uniform(8, 25)
    ang = rng.uniform(-0.6, 0.6) + math.pi
    eye = np.array([dist * math.sin(ang), rng.uniform(1.5, 8), dist * math.cos(ang)])
    target = np.array([rng.uniform(-4, 4), rng.uniform(0, 2), rng.uniform(-2, 4)])
    lens = 0.0 if rng.random() < 0.6 else rng.uniform(0.01, 0.05)
    fov = float(np.exp(rng.uniform(math.log(8), math.log(60))))
    return {"position": tuple(-eye), "lookdir": tuple(eye - target), "fov_degrees": fov,
            "lens_radius": lens, "focus_dist": float(np.linalg.norm(eye - target))}
