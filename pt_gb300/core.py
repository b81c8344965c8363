"""Python host mirror of the reference's path-tracing operator interface.

`PathTraceDispatcher(scene, width, height).start(params)` mirrors
src/pathtrace/ptdispatch.h:13-33 (constructor + start) and produces the same
output file and stdout lines as `pt --headless`; `Context` is the thin
object wrapper of the C ABI in include/pt_gpu.h; `HostScene` wraps the scene
front end of include/pt_scene.h.  Every call goes through libptgpu.so; there
is no Python or CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import abi
from .abi import lib, PtError


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class HostScene:
    """A scene on the host: parsed .scn + glTF, or raw arrays; packs to the device layout."""

    def __init__(self, handle: int):
        if not handle:
            raise PtError(abi.PT_ERR_INVALID, lib().pt_scene_last_error().decode())
        self._h = C.c_void_p(handle)
        self._view = None

    @classmethod
    def load(cls, scn_path: str | Path) -> "HostScene":
        return cls(lib().pt_scene_load(str(scn_path).encode()))

    @classmethod
    def from_raw(cls, raw: dict, camera: dict | None = None) -> "HostScene":
        """raw: dict of numpy arrays (see raw_to_struct); copied by the library."""
        rs, keep = raw_to_struct(raw)
        cam = camera_struct(camera) if camera is not None else None
        h = lib().pt_scene_from_raw(C.byref(rs), C.byref(cam) if cam is not None else None)
        del keep
        return cls(h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().pt_scene_free(h)
            self._h = C.c_void_p(0)

    def raw(self) -> dict:
        rs = abi.RawScene()
        _check(lib().pt_scene_raw(self._h, C.byref(rs)), None)
        return struct_to_raw(rs)

    def camera(self) -> abi.CameraDesc:
        cd = abi.CameraDesc()
        _check(lib().pt_scene_camera(self._h, C.byref(cd)), None)
        return cd

    def pack(self) -> abi.SceneView:
        v = abi.SceneView()
        rc = lib().pt_scene_pack(self._h, C.byref(v))
        if rc != abi.PT_OK:
            raise PtError(rc, lib().pt_scene_last_error().decode())
        self._view = v
        return v

    def details(self) -> str:
        buf = C.create_string_buffer(2048)
        _check(lib().pt_scene_details(self._h, buf, len(buf)), None)
        return buf.value.decode()

    def render_params(self, width: int, height: int, samples: int, max_bounces: int, sample_index: int = 0,
                      accum_mode: int = abi.PT_ACCUM_FP32, kernel: int = abi.PT_KERNEL_AUTO,
                      rr_start: int = 1) -> abi.RenderParams:
        p = abi.RenderParams()
        cam = self.camera()
        _check(lib().pt_camera_params(C.byref(cam), width, height, C.byref(p)), None)
        p.sample_index = sample_index
        p.samples = samples
        p.max_bounces = max_bounces
        p.accum_mode = accum_mode
        p.kernel = kernel
        p.rr_start = rr_start
        return p


def _check(rc: int, ctx) -> None:
    if rc != abi.PT_OK:
        msg = lib().pt_last_error(ctx).decode() if ctx is not None else lib().pt_scene_last_error().decode()
        raise PtError(rc, msg)


class Context:
    """One device context (pt_ctx) on CUDA device `device`."""

    def __init__(self, device: int = 0):
        h = lib().pt_create(device)
        if not h:
            raise PtError(abi.PT_ERR_CUDA, lib().pt_last_error(None).decode())
        self._h = C.c_void_p(h)
        self.width = 0
        self.height = 0

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().pt_destroy(self._h)
            self._h = C.c_void_p(0)

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, view: abi.SceneView) -> None:
        _check(lib().pt_upload_scene(self._h, C.byref(view)), self._h)

    def build_accel(self) -> abi.AccelInfo:
        info = abi.AccelInfo()
        _check(lib().pt_build_accel(self._h, C.byref(info)), self._h)
        return info

    def render(self, params: abi.RenderParams, stats: bool = True):
        st = abi.RenderStats()
        _check(lib().pt_render(self._h, C.byref(params), C.byref(st) if stats else None), self._h)
        self.width, self.height = params.width, params.height
        return st if stats else None

    def set_camera(self, params: abi.RenderParams) -> None:
        """Keeps camera and image settings and restarts accumulation (PathTracer::set_camera)."""
        _check(lib().pt_set_camera(self._h, C.byref(params)), self._h)
        self.width, self.height = params.width, params.height

    def render_next(self, samples: int = 1, stats: bool = True):
        """Adds `samples` samples to the running mean of the set camera."""
        st = abi.RenderStats()
        _check(lib().pt_render_next(self._h, samples, C.byref(st) if stats else None), self._h)
        return st if stats else None

    def synchronize(self) -> None:
        _check(lib().pt_synchronize(self._h), self._h)

    def tonemap(self) -> None:
        _check(lib().pt_tonemap(self._h), self._h)

    def read_image(self, fp64: bool = False, out: np.ndarray | None = None) -> np.ndarray:
        dt = np.float64 if fp64 else np.float32
        if out is None:
            out = np.empty((self.height, self.width, 4), dtype=dt)
        _check(lib().pt_read_image(self._h, out.ctypes.data, out.strides[0], 1 if fp64 else 0), self._h)
        return out

    def restore_image(self, rgba: np.ndarray, samples_done: int, sums64: np.ndarray | None = None) -> None:
        """Puts a checkpoint (read_image(), and read_image sums for FP64
        renders) back; render from sample_index = samples_done to resume."""
        img = np.ascontiguousarray(rgba, np.float32)
        h, w = img.shape[:2]
        s64 = None if sums64 is None else np.ascontiguousarray(sums64, np.float64)
        _check(lib().pt_restore_image(self._h, _ptr(img, C.c_float), img.strides[0],
                                      None if s64 is None else _ptr(s64, C.c_double), w, h, samples_done), self._h)
        self.width, self.height = w, h

    def read_denoised(self, out: np.ndarray | None = None) -> np.ndarray:
        """The image of the last denoise() (RGBA float32)."""
        if out is None:
            out = np.empty((self.height, self.width, 4), dtype=np.float32)
        _check(lib().pt_read_image(self._h, out.ctypes.data, out.strides[0], abi.PT_IMAGE_DENOISED), self._h)
        return out

    def render_features(self, params: abi.RenderParams) -> None:
        """First-hit albedo / normal / depth of the camera rays of `params`' samples."""
        _check(lib().pt_render_features(self._h, C.byref(params)), self._h)

    def read_features(self):
        """(albedo + hit distance, shading normal) of the last features, [h, w, 4] float32 each."""
        a = np.empty((self.height, self.width, 4), np.float32)
        n = np.empty_like(a)
        _check(lib().pt_read_features(self._h, a.ctypes.data, n.ctypes.data), self._h)
        return a, n

    def denoise_snapshot(self) -> None:
        """Keeps the current mean image; the denoiser input then carries a noise estimate."""
        _check(lib().pt_denoise_snapshot(self._h), self._h)

    def render_noisy(self, params: abi.RenderParams) -> None:
        """The denoiser's input side in one render: params.samples samples with
        the first-hit features of every sample (PT_RENDER_FEATURES) and a
        snapshot armed at half of them (the noise estimate)."""
        s, flags = params.samples, params.flags
        try:
            if s >= 2:
                _check(lib().pt_denoise_snapshot_at(self._h, params.sample_index + s // 2), self._h)
            params.flags = flags | abi.PT_RENDER_FEATURES
            self.render(params, stats=False)
        finally:
            params.flags = flags

    def render_denoised(self, unet, params: abi.RenderParams) -> None:
        """render_noisy, then the network; read the result with read_denoised()."""
        self.render_noisy(params)
        self.denoise(unet, params.samples)

    def denoise_input(self, spp: int, dst_ptr: int, base_ptr: int | None = None) -> None:
        """Packs the current image and features into a bf16 [h, w, 16] device
        buffer (and the fp32 [h, w, 4] residual base when base_ptr is given)."""
        _check(lib().pt_denoise_input(self._h, spp, dst_ptr, base_ptr, None), self._h)

    def denoise(self, unet, spp: int) -> None:
        """Runs `unet` (a pt_gb300.denoise.UNet of batch 1 and this image's size)."""
        _check(lib().pt_denoise(self._h, unet.handle, spp), self._h)

    def mse(self, reference: np.ndarray) -> float:
        ref = np.ascontiguousarray(reference, dtype=np.float32)
        v = C.c_double()
        _check(lib().pt_mse_host(self._h, _ptr(ref, C.c_float), C.byref(v)), self._h)
        return v.value

    def render_batch(self, jobs, flags: int = 0) -> abi.BatchStats:
        """Render [(scene Context, RenderParams), ...] as one batch (pt_render_batch)."""
        arr = (abi.BatchJob * len(jobs))()
        for i, (ctx, params) in enumerate(jobs):
            arr[i].scene = ctx._h.value
            arr[i].params = params
        st = abi.BatchStats()
        _check(lib().pt_render_batch(self._h, arr, len(jobs), flags, C.byref(st)), self._h)
        self._batch_sizes = [(p.height, p.width) for _, p in jobs]
        return st

    def batch_job_times(self) -> np.ndarray:
        """Per-job completion times (ms from the start) of the last render_batch."""
        n = len(self._batch_sizes)
        out = np.zeros(n, np.float32)
        _check(lib().pt_batch_job_times(self._h, _ptr(out, C.c_float), n), self._h)
        return out

    def read_batch_image(self, job: int, fp64: bool = False) -> np.ndarray:
        h, w = self._batch_sizes[job]
        out = np.empty((h, w, 4), dtype=np.float64 if fp64 else np.float32)
        _check(lib().pt_read_batch_image(self._h, job, out.ctypes.data, out.strides[0], 1 if fp64 else 0), self._h)
        return out


@dataclass
class PathTraceParameters:
    """The reference's PathTraceParameters (ptdispatch.h:12-20)."""
    out_path: str
    output_format: str = "png"  # "png" or "hdr"
    samples: int = 32
    max_bounces: int = 2
    render_time: float = float("inf")  # parsed but unused, as in the reference


class PathTraceDispatcher:
    """Headless renderer with the reference's interface (ptdispatch.cpp:18-95)."""

    def __init__(self, scene: HostScene, width: int, height: int, device: int = 0):
        self.scene = scene
        self.width = width
        self.height = height
        self.ctx = Context(device)
        self.ctx.upload(scene.pack())
        self.accel = self.ctx.build_accel()

    def start(self, params: PathTraceParameters) -> np.ndarray:
        fmt = params.output_format.lower()
        if fmt not in ("png", "hdr"):
            raise PtError(abi.PT_ERR_INVALID, "No output format was given.")
        if params.samples == 0:
            raise PtError(abi.PT_ERR_INVALID, "Sample count is zero.")
        rp = self.scene.render_params(self.width, self.height, params.samples, params.max_bounces)
        t0 = time.perf_counter()
        self.ctx.render(rp, stats=False)
        if fmt == "png":
            self.ctx.tonemap()
        img = self.ctx.read_image()
        taken = time.perf_counter() - t0
        print(f"Rendering took {taken:g} seconds with {params.samples} samples taken per pixel.")
        print(f"{params.samples / taken:g} samples per second.")
        print(f"Writing image to {params.out_path}")
        write = lib().pt_write_png if fmt == "png" else lib().pt_write_hdr
        flat = np.ascontiguousarray(img)
        rc = write(params.out_path.encode(), _ptr(flat, C.c_float), self.width, self.height)
        if rc != abi.PT_OK:
            raise PtError(rc, f"Could not write {fmt.upper()} file.")
        return img


# ---------------------------------------------------------------- raw scene helpers

def raw_to_struct(raw: dict):
    """numpy dict -> RawScene; returns (struct, keep-alive list)."""
    keep = []

    def arr(name, dtype, shape_tail=None):
        a = np.ascontiguousarray(raw.get(name, np.zeros((0,) + (shape_tail or ()), dtype)), dtype=dtype)
        keep.append(a)
        return a

    v = arr("vertices", np.float32)
    idx = arr("indices", np.uint32)
    meshes = arr("meshes", np.uint32)
    mm = arr("mesh_material", np.uint32)
    mio = arr("mesh_instance_offset", np.uint32)
    im = arr("instance_matrices", np.float32)
    mats = arr("materials", np.float32)
    pl = arr("point_lights", np.float32)
    dl = arr("directional_lights", np.float32)
    rs = abi.RawScene()
    rs.vertices = _ptr(v, C.c_float)
    rs.vertex_count = v.size // abi.PT_VERTEX_FLOATS
    rs.indices = _ptr(idx, C.c_uint32)
    rs.index_count = idx.size
    rs.meshes = meshes.ctypes.data_as(C.POINTER(abi.MeshRange))
    rs.mesh_material = _ptr(mm, C.c_uint32)
    rs.mesh_instance_offset = _ptr(mio, C.c_uint32)
    rs.mesh_count = mm.size
    rs.instance_matrices = _ptr(im, C.c_float)
    rs.instance_count = im.size // 16
    rs.materials = mats.ctypes.data_as(C.POINTER(abi.Material))
    rs.material_count = mats.size // 24
    rs.point_lights = _ptr(pl, C.c_float)
    rs.point_light_count = pl.size // 6
    rs.directional_lights = _ptr(dl, C.c_float)
    rs.directional_light_count = dl.size // 6
    env = raw.get("environment_colour", (0.0, 0.0, 0.0))
    for k in range(3):
        rs.environment_colour[k] = float(env[k])
    # textures: raw["textures"] = [(uint8 array [h, w, c], srgb)], c in 1, 2, 4
    texs = raw.get("textures", [])
    if texs:
        parts, descs, off = [], (abi.Texture * len(texs))(), 0
        for i, (img, srgb) in enumerate(texs):
            img = np.ascontiguousarray(img, dtype=np.uint8)
            h, w = img.shape[:2]
            c = 1 if img.ndim == 2 else img.shape[2]
            descs[i].offset, descs[i].width, descs[i].height, descs[i].channels, descs[i].srgb = off, w, h, c, int(srgb)
            parts.append(img.reshape(-1))
            off += img.size
        texels = np.ascontiguousarray(np.concatenate(parts))
        keep += [texels, descs]
        rs.texels = _ptr(texels, C.c_uint8)
        rs.texel_bytes = texels.size
        rs.textures = descs
        rs.texture_count = len(texs)
    # refractive extension: raw["material_ior"] = float per material (0 = the reference's BSDF)
    if raw.get("material_ior") is not None:
        ior = np.ascontiguousarray(raw["material_ior"], np.float32).reshape(-1)
        if ior.size != rs.material_count:
            raise ValueError("material_ior needs one entry per material")
        keep.append(ior)
        rs.material_ior = _ptr(ior, C.c_float)
    return rs, keep


def struct_to_raw(rs: abi.RawScene) -> dict:
    def a(ptr, n, dtype):
        if n == 0:
            return np.zeros(0, dtype)
        return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)

    return {
        "vertices": a(rs.vertices, rs.vertex_count * abi.PT_VERTEX_FLOATS, np.float32).reshape(-1, 8),
        "indices": a(rs.indices, rs.index_count, np.uint32),
        "meshes": a(C.cast(rs.meshes, C.POINTER(C.c_uint32)), rs.mesh_count * 4, np.uint32).reshape(-1, 4),
        "mesh_material": a(rs.mesh_material, rs.mesh_count, np.uint32),
        "mesh_instance_offset": a(rs.mesh_instance_offset, rs.mesh_count + 1, np.uint32),
        "instance_matrices": a(rs.instance_matrices, rs.instance_count * 16, np.float32).reshape(-1, 16),
        "materials": a(C.cast(rs.materials, C.POINTER(C.c_float)), rs.material_count * 24, np.float32).reshape(-1, 24),
        "point_lights": a(rs.point_lights, rs.point_light_count * 6, np.float32).reshape(-1, 6),
        "directional_lights": a(rs.directional_lights, rs.directional_light_count * 6, np.float32).reshape(-1, 6),
        "environment_colour": np.array(list(rs.environment_colour), np.float32),
        "textures": [(np.ctypeslib.as_array(rs.texels, shape=(rs.texel_bytes,))[
                          t.offset:t.offset + t.width * t.height * t.channels].reshape(
                          (t.height, t.width) if t.channels == 1 else (t.height, t.width, t.channels)).copy(), bool(t.srgb))
                     for t in (rs.textures[i] for i in range(rs.texture_count))],
        "material_ior": a(rs.material_ior, rs.material_count, np.float32) if rs.material_ior else None,
    }


def camera_struct(cam: dict) -> abi.CameraDesc:
    cd = abi.CameraDesc()
    d = {"position": (0, 0, 0), "lookdir": (0, 0, -1), "up": (0, 1, 0), "fov_degrees": 45.0, "near_plane": 0.1,
         "far_plane": 1000.0, "focus_dist": 0.0, "lens_radius": 0.0, "exposure": 1.0}
    d.update(cam)
    for k in ("position", "lookdir", "up"):
        for i in range(3):
            getattr(cd, k)[i] = float(d[k][i])
    for k in ("fov_degrees", "near_plane", "far_plane", "focus_dist", "lens_radius", "exposure"):
        setattr(cd, k, float(d[k]))
    return cd


def view_arrays(v: abi.SceneView) -> dict:
    """Copy the arrays of a packed scene view into numpy (for comparisons)."""
    def a(ptr, n, dtype):
        if n == 0 or not ptr:
            return np.zeros(0, dtype)
        return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)

    return {
        "vertices": a(v.vertices, v.vertex_count * 8, np.float32),
        "indices": a(v.indices, v.index_count, np.uint32),
        "meshes": a(C.cast(v.meshes, C.POINTER(C.c_uint32)), v.mesh_count * 4, np.uint32),
        "instances": a(C.cast(v.instances, C.POINTER(C.c_uint32)), v.instance_count * 32, np.uint32),
        "instance_mesh": a(v.instance_mesh, v.instance_count, np.uint32),
        "w2o": a(v.instance_world_to_object, v.instance_count * 12, np.float32),
        "opaque": a(v.instance_opaque, v.instance_count, np.uint8),
        "materials": a(C.cast(v.materials, C.POINTER(C.c_uint32)), v.material_count * 24, np.uint32),
        "light": a(v.light_words, v.light_word_count, np.uint32),
        "light_count": v.light_count,
        "env": np.array(list(v.environment_colour), np.float32),
        "texels": a(v.texels, v.texel_bytes, np.uint8),
        "textures": a(C.cast(v.textures, C.POINTER(C.c_uint32)), v.texture_count * 6, np.uint32),
        "material_ior": a(v.material_ior, v.material_count, np.float32),
    }
