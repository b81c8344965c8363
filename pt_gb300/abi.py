"""ctypes mirror of include/pt_gpu.h and include/pt_scene.h, and the loader
of libptgpu.so.

The library is loaded lazily on first use.  There is no fallback: if the
native library is missing or cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_HERE = Path(__file__).resolve().parent
# PT_CHECKED=1 selects the bounds-checked build of the same library
LIB_PATH = _HERE / "_build" / ("libptgpu_checked.so" if os.environ.get("PT_CHECKED") == "1" else "libptgpu.so")
ABI_VERSION = 2  # PT_ABI_VERSION of include/pt_gpu.h that these declarations follow

PT_OK = 0
PT_ERR_INVALID = -1
PT_ERR_CUDA = -2
PT_ERR_OOM = -3
PT_ERR_STATE = -4
PT_ERR_TIMEOUT = -5
PT_ERR_DEVICE = -6
PT_ERR_IO = -7
PT_ERR_UNSUPPORTED = -8
STATUS_NAMES = {0: "PT_OK", -1: "PT_ERR_INVALID", -2: "PT_ERR_CUDA", -3: "PT_ERR_OOM", -4: "PT_ERR_STATE",
                -5: "PT_ERR_TIMEOUT", -6: "PT_ERR_DEVICE", -7: "PT_ERR_IO", -8: "PT_ERR_UNSUPPORTED"}

PT_ACCUM_FP32 = 0
PT_ACCUM_FP32_FP64 = 1
PT_KERNEL_AUTO = 0
PT_KERNEL_MEGA = 1
PT_KERNEL_WAVEFRONT = 2

PT_VERTEX_FLOATS = 8
PT_NO_EMITTER_INDEX = 0xFFFFFFFF
PT_BASE_COLOUR_MAP_BIT = 1 << 0
PT_EMISSION_MAP_BIT = 1 << 1
PT_ROUGHNESS_MAP_BIT = 1 << 2
PT_METALNESS_MAP_BIT = 1 << 3
PT_ROUGHNESS_METALNESS_MAP_BIT = 1 << 4
PT_SPECULAR_MAP_BIT = 1 << 5
PT_SHEEN_MAP_BIT = 1 << 7
PT_CLEARCOAT_MAP_BIT = 1 << 9
PT_NORMAL_MAP_BIT = 1 << 12
PT_MATERIAL_IS_TRANSPARENT_BIT = 1 << 13


class MeshRange(C.Structure):
    _fields_ = [("vertex_offset", C.c_uint32), ("index_offset", C.c_uint32), ("tri_count", C.c_uint32),
                ("vertex_count", C.c_uint32)]


class InstanceData(C.Structure):
    _fields_ = [("vertex_index", C.c_uint32), ("index_index", C.c_uint32), ("emitter_index", C.c_uint32),
                ("material_index", C.c_uint32), ("transform", (C.c_float * 4) * 4), ("normal", (C.c_float * 4) * 3)]


class Material(C.Structure):
    _fields_ = [("base_colour", C.c_float * 4), ("emission", C.c_float * 4),
                ("rough_metal_normal_map_bits", C.c_float * 4), ("specular", C.c_float * 4),
                ("sheen", C.c_float * 4), ("cc_ccrgh_aniso", C.c_float * 4)]


class Texture(C.Structure):
    _fields_ = [("offset", C.c_uint64), ("width", C.c_uint32), ("height", C.c_uint32), ("channels", C.c_uint32),
                ("srgb", C.c_uint32)]


class SceneView(C.Structure):
    _fields_ = [("vertices", C.POINTER(C.c_float)), ("vertex_count", C.c_uint32),
                ("indices", C.POINTER(C.c_uint32)), ("index_count", C.c_uint32),
                ("meshes", C.POINTER(MeshRange)), ("mesh_count", C.c_uint32),
                ("instances", C.POINTER(InstanceData)), ("instance_mesh", C.POINTER(C.c_uint32)),
                ("instance_world_to_object", C.POINTER(C.c_float)), ("instance_opaque", C.POINTER(C.c_uint8)),
                ("instance_count", C.c_uint32),
                ("materials", C.POINTER(Material)), ("material_count", C.c_uint32),
                ("light_words", C.POINTER(C.c_uint32)), ("light_word_count", C.c_uint32), ("light_count", C.c_uint32),
                ("environment_colour", C.c_float * 3),
                ("texels", C.POINTER(C.c_uint8)), ("texel_bytes", C.c_uint64), ("textures", C.POINTER(Texture)),
                ("texture_count", C.c_uint32), ("material_ior", C.POINTER(C.c_float))]


class RenderParams(C.Structure):
    _fields_ = [("inv_view", C.c_float * 16), ("inv_proj", C.c_float * 16), ("near_plane", C.c_float),
                ("far_plane", C.c_float), ("focus_dist", C.c_float), ("lens_radius", C.c_float),
                ("exposure", C.c_float), ("width", C.c_uint32), ("height", C.c_uint32),
                ("sample_index", C.c_uint32), ("samples", C.c_uint32), ("max_bounces", C.c_uint32),
                ("accum_mode", C.c_uint32), ("kernel", C.c_uint32), ("rr_start", C.c_uint32),
                ("flags", C.c_uint32), ("reserved", C.c_uint32 * 2)]


class RenderStats(C.Structure):
    _fields_ = [("segments", C.c_uint64), ("shadow_rays", C.c_uint64), ("paths", C.c_uint64),
                ("node_visits", C.c_uint64), ("tri_tests", C.c_uint64), ("milliseconds", C.c_float),
                ("kernel_launches", C.c_uint32), ("kernel_used", C.c_uint32), ("error_word", C.c_uint32),
                ("stage_ms", C.c_float * 6), ("stage_launches", C.c_uint32)]


STAGES = ("raygen", "extend", "shade", "shadow", "reset", "accumulate")


class BatchJob(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("params", RenderParams)]


class BatchStats(C.Structure):
    _fields_ = [("segments", C.c_uint64), ("shadow_rays", C.c_uint64), ("paths", C.c_uint64),
                ("milliseconds", C.c_float), ("tune_milliseconds", C.c_float), ("build_milliseconds", C.c_float),
                ("waves", C.c_uint32), ("kernel_launches", C.c_uint32), ("mega_jobs", C.c_uint32),
                ("wave_capacity", C.c_uint32), ("tile_w", C.c_uint32), ("graph_reused", C.c_uint32),
                ("mega_threshold", C.c_uint64), ("error_word", C.c_uint32), ("reserved", C.c_uint32)]


PT_BATCH_NO_TUNE = 1
PT_BATCH_NO_GRAPH = 2
PT_BATCH_RETUNE = 4


def PT_BATCH_CAPACITY_LOG2(n: int) -> int:
    return n << 8


class AccelInfo(C.Structure):
    _fields_ = [("blas_count", C.c_uint32), ("tlas_nodes", C.c_uint32), ("blas_nodes", C.c_uint64),
                ("triangles", C.c_uint64), ("device_bytes", C.c_uint64), ("build_ms", C.c_float)]


class RawScene(C.Structure):
    _fields_ = [("vertices", C.POINTER(C.c_float)), ("vertex_count", C.c_uint32),
                ("indices", C.POINTER(C.c_uint32)), ("index_count", C.c_uint32),
                ("meshes", C.POINTER(MeshRange)), ("mesh_material", C.POINTER(C.c_uint32)),
                ("mesh_instance_offset", C.POINTER(C.c_uint32)), ("mesh_count", C.c_uint32),
                ("instance_matrices", C.POINTER(C.c_float)), ("instance_count", C.c_uint32),
                ("materials", C.POINTER(Material)), ("material_count", C.c_uint32),
                ("point_lights", C.POINTER(C.c_float)), ("point_light_count", C.c_uint32),
                ("directional_lights", C.POINTER(C.c_float)), ("directional_light_count", C.c_uint32),
                ("environment_colour", C.c_float * 3),
                ("texels", C.POINTER(C.c_uint8)), ("texel_bytes", C.c_uint64), ("textures", C.POINTER(Texture)),
                ("texture_count", C.c_uint32), ("material_ior", C.POINTER(C.c_float))]


class CameraDesc(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("lookdir", C.c_float * 3), ("up", C.c_float * 3),
                ("fov_degrees", C.c_float), ("near_plane", C.c_float), ("far_plane", C.c_float),
                ("focus_dist", C.c_float), ("lens_radius", C.c_float), ("exposure", C.c_float)]


# (name, restype, argtypes) of every entry point declared in include/*.h
SIGNATURES = [
    ("pt_abi_version", C.c_int, []),
    ("pt_create", C.c_void_p, [C.c_int]),
    ("pt_destroy", None, [C.c_void_p]),
    ("pt_last_error", C.c_char_p, [C.c_void_p]),
    ("pt_upload_scene", C.c_int, [C.c_void_p, C.POINTER(SceneView)]),
    ("pt_build_accel", C.c_int, [C.c_void_p, C.POINTER(AccelInfo)]),
    ("pt_render", C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.POINTER(RenderStats)]),
    ("pt_set_camera", C.c_int, [C.c_void_p, C.POINTER(RenderParams)]),
    ("pt_render_next", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(RenderStats)]),
    ("pt_read_image", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]),
    ("pt_synchronize", C.c_int, [C.c_void_p]),
    ("pt_restore_image", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_size_t, C.POINTER(C.c_double), C.c_uint32,
                                   C.c_uint32, C.c_uint32]),
    ("pt_tonemap", C.c_int, [C.c_void_p]),
    ("pt_mse_host", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_double)]),
    ("pt_mse_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]),
    ("pt_render_batch", C.c_int, [C.c_void_p, C.POINTER(BatchJob), C.c_uint32, C.c_uint32, C.POINTER(BatchStats)]),
    ("pt_batch_job_times", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_uint32]),
    ("pt_read_batch_image", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_size_t, C.c_int]),
    ("pt_scene_last_error", C.c_char_p, []),
    ("pt_scene_load", C.c_void_p, [C.c_char_p]),
    ("pt_scene_from_raw", C.c_void_p, [C.POINTER(RawScene), C.POINTER(CameraDesc)]),
    ("pt_scene_free", None, [C.c_void_p]),
    ("pt_scene_raw", C.c_int, [C.c_void_p, C.POINTER(RawScene)]),
    ("pt_scene_camera", C.c_int, [C.c_void_p, C.POINTER(CameraDesc)]),
    ("pt_scene_pack", C.c_int, [C.c_void_p, C.POINTER(SceneView)]),
    ("pt_camera_params", C.c_int, [C.POINTER(CameraDesc), C.c_uint32, C.c_uint32, C.POINTER(RenderParams)]),
    ("pt_from_srgb", C.c_float, [C.c_float]),
    ("pt_scene_details", C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    ("pt_write_hdr", C.c_int, [C.c_char_p, C.POINTER(C.c_float), C.c_uint32, C.c_uint32]),
    ("pt_write_png", C.c_int, [C.c_char_p, C.POINTER(C.c_float), C.c_uint32, C.c_uint32]),
    ("pt_read_hdr", C.c_int, [C.c_char_p, C.POINTER(C.POINTER(C.c_float)), C.POINTER(C.c_uint32),
                              C.POINTER(C.c_uint32)]),
    ("pt_host_free", None, [C.c_void_p]),
    ("pt_png_decode", C.c_int, [C.c_void_p, C.c_size_t, C.POINTER(C.POINTER(C.c_uint8)), C.POINTER(C.c_uint32),
                                C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    ("pt_jpeg_decode", C.c_int, [C.c_void_p, C.c_size_t, C.POINTER(C.POINTER(C.c_uint8)), C.POINTER(C.c_uint32),
                                C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    # denoiser (include/pt_denoise.h)
    ("pt_debug_poke_tlas_link", C.c_int, [C.c_void_p, C.c_int]),
    ("pt_unet_param_count", C.c_size_t, []),
    ("pt_unet_layer_shape", C.c_int, [C.c_int, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    ("pt_unet_create", C.c_void_p, [C.c_int, C.c_uint32, C.c_uint32, C.c_uint32]),
    ("pt_unet_destroy", None, [C.c_void_p]),
    ("pt_unet_last_error", C.c_char_p, [C.c_void_p]),
    ("pt_unet_set_params", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_size_t]),
    ("pt_unet_get_params", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_size_t]),
    ("pt_unet_get_grads", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_size_t]),
    ("pt_unet_shape", None, [C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    ("pt_unet_input", C.c_void_p, [C.c_void_p]),
    ("pt_unet_output", C.c_void_p, [C.c_void_p]),
    ("pt_unet_base", C.c_void_p, [C.c_void_p]),
    ("pt_unet_forward", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("pt_unet_backward", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_double), C.c_void_p]),
    ("pt_unet_adam", C.c_int, [C.c_void_p, C.c_float, C.c_void_p]),
    ("pt_unet_get_adam_state", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_size_t,
                                         C.POINTER(C.c_uint32)]),
    ("pt_unet_set_adam_state", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_size_t,
                                         C.c_uint32]),
    ("pt_nn_conv3x3", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p, C.c_void_p]),
    ("pt_nn_conv3x3_dgrad", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32,
                                      C.c_void_p, C.c_void_p, C.c_void_p]),
    ("pt_nn_conv3x3_wgrad", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                      C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    ("pt_render_features", C.c_int, [C.c_void_p, C.POINTER(RenderParams)]),
    ("pt_read_features", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("pt_denoise_snapshot", C.c_int, [C.c_void_p]),
    ("pt_denoise_snapshot_at", C.c_int, [C.c_void_p, C.c_uint32]),
    ("pt_denoise_input", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("pt_denoise", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
]

PT_IMAGE_DENOISED = 2
PT_RENDER_FEATURES = 1
PT_RENDER_TIME_STAGES = 2
PT_RENDER_FEATURES_FP16 = 4
PT_RENDER_RESTART = 8
PT_IMAGE_SUMS64 = 3
PT_UNET_IN_CHANNELS = 16
PT_UNET_OUT_CHANNELS = 16

_lib = None


class NativeLibraryMissing(RuntimeError):
    pass


def lib():
    """Load libptgpu.so (built by pt_gb300.build) and declare its signatures."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise NativeLibraryMissing(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "or `python pt_gb300/build.py`")
        L = C.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        if L.pt_abi_version() != ABI_VERSION:
            raise NativeLibraryMissing(f"{LIB_PATH} has ABI version {L.pt_abi_version()}, these bindings "
                                       f"expect {ABI_VERSION}: rebuild it")
        _lib = L
    return _lib


class PtError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
