"""Python binding of the CPU oracle (oracle/_build/liboracle.so) and of the
reference's own CPU code compiled here (oracle/_ref/libptref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference legs, never by the product (pt_gb300).
The oracle is the checker of the CUDA path: see oracle/pt_oracle.h for the
reference functions it restates and how each is pinned.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libptref.so"
REF_MEANSQ = HERE / "_ref" / "meansq"
# Where the reference's source tree is read from (its CPU sources for
# oracle/_ref, one shader table as text for the golden fixtures): the one
# setting of that location, PT_REFERENCE_TREE, with the tree's usual place as
# the default.  Where no tree exists (the GPU machine) everything that needs
# it is skipped.
_DEFAULT_REFERENCE_TREE = "/root/reference"


def reference_tree() -> Path | None:
    """The reference's source tree, or None where it does not exist."""
    p = Path(os.environ.get("PT_REFERENCE_TREE", _DEFAULT_REFERENCE_TREE))
    return p if (p / "src").is_dir() else None


def build(reference: bool | None = None) -> None:
    """Compile the oracle (and the reference shim when the reference tree exists)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "oracle"], check=True)
    tree = reference_tree()
    if reference is None:
        reference = tree is not None
    if reference:
        if tree is None:
            raise FileNotFoundError("no reference tree (set PT_REFERENCE_TREE)")
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={tree}"], check=True)


_lib = None
_ref = None


class OrStats(C.Structure):
    _fields_ = [("segments", C.c_uint64), ("shadow_rays", C.c_uint64), ("paths", C.c_uint64),
                ("node_visits", C.c_uint64), ("tri_tests", C.c_uint64), ("inst_visits", C.c_uint64),
                ("ray_count", C.c_uint64)]


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build(reference=False)
        from pt_gb300 import abi  # struct layouts of the C ABI (include/pt_gpu.h)
        L = C.CDLL(str(LIB))
        L.or_hash.restype = C.c_uint32
        L.or_hash.argtypes = [C.c_uint32]
        L.or_hash_combine.restype = C.c_uint32
        L.or_hash_combine.argtypes = [C.c_uint32, C.c_uint32]
        L.or_sobol.restype = C.c_uint32
        L.or_sobol.argtypes = [C.c_uint32, C.c_uint32]
        L.or_scramble.restype = C.c_uint32
        L.or_scramble.argtypes = [C.c_uint32, C.c_uint32]
        L.or_sampler_sequence.restype = C.c_uint32
        L.or_sampler_sequence.argtypes = [C.c_uint32] * 4 + [C.POINTER(C.c_uint8), C.c_uint32, C.POINTER(C.c_float)]
        L.or_sin.restype = C.c_float
        L.or_sin.argtypes = [C.c_float]
        L.or_cos.restype = C.c_float
        L.or_cos.argtypes = [C.c_float]
        L.or_xshiro128_stream.argtypes = [C.POINTER(C.c_uint32), C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_float)]
        L.or_splitmix32_stream.argtypes = [C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32)]
        L.or_alias_build.argtypes = [C.POINTER(C.c_float), C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                     C.POINTER(C.c_uint32)]
        L.or_from_srgb.restype = C.c_float
        L.or_from_srgb.argtypes = [C.c_float]
        L.or_camera_params.argtypes = [C.POINTER(abi.CameraDesc), C.c_uint32, C.c_uint32, C.POINTER(abi.RenderParams)]
        L.or_pack.restype = C.c_void_p
        L.or_pack.argtypes = [C.POINTER(abi.RawScene)]
        L.or_packed_view.argtypes = [C.c_void_p, C.POINTER(abi.SceneView)]
        L.or_packed_free.argtypes = [C.c_void_p]
        L.or_scene_create.restype = C.c_void_p
        L.or_scene_create.argtypes = [C.POINTER(abi.SceneView), C.c_int]
        L.or_scene_destroy.argtypes = [C.c_void_p]
        L.or_texture_sample.argtypes = [C.c_void_p, C.c_uint32, C.c_float, C.c_float, C.POINTER(C.c_float)]
        L.or_render.restype = C.c_int
        L.or_render.argtypes = [C.c_void_p, C.POINTER(abi.RenderParams), C.c_uint32, C.c_uint32, C.POINTER(C.c_float),
                                C.POINTER(C.c_double), C.POINTER(OrStats), C.c_int]
        L.or_path_signature.restype = C.c_uint32
        L.or_path_signature.argtypes = [C.c_void_p, C.POINTER(abi.RenderParams), C.c_uint32, C.c_uint32, C.c_uint32,
                                        C.POINTER(C.c_uint64), C.c_uint32]
        L.or_intersect.restype = C.c_int
        L.or_intersect.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float, C.c_float,
                                   C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                   C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.or_meansq.restype = C.c_double
        L.or_meansq.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint32, C.c_uint32]
        L.or_meansq64.restype = C.c_double
        L.or_meansq64.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_float), C.c_uint32, C.c_uint32]
        L.or_max_threads.restype = C.c_int
        L.or_tonemap.argtypes = [C.POINTER(C.c_float), C.c_uint64]
        _lib = L
    return _lib


def ref():
    """The reference's own CPU code (only where the reference tree was compiled)."""
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            return None
        from pt_gb300 import abi
        R = C.CDLL(str(REF_LIB))
        R.ref_xshiro128_stream.argtypes = [C.POINTER(C.c_uint32), C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_float)]
        R.ref_splitmix32_stream.argtypes = [C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32)]
        R.ref_alias_build.argtypes = [C.POINTER(C.c_float), C.c_uint32, C.POINTER(C.c_uint32)]
        R.ref_from_srgb.restype = C.c_float
        R.ref_from_srgb.argtypes = [C.c_float]
        R.ref_camera_params.argtypes = [C.POINTER(abi.CameraDesc), C.c_uint32, C.c_uint32, C.POINTER(C.c_float),
                                        C.POINTER(C.c_float)]
        R.ref_instance_matrices.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)]
        R.ref_light_stream.restype = C.c_int
        R.ref_light_stream.argtypes = [C.POINTER(abi.RawScene), C.POINTER(C.c_uint32), C.c_uint32, C.POINTER(C.c_uint32)]
        R.ref_is_emitter.restype = C.c_int
        R.ref_is_emitter.argtypes = [C.POINTER(abi.Material)]
        R.ref_parse_transform.restype = C.c_int
        R.ref_parse_transform.argtypes = [C.c_char_p, C.POINTER(C.c_float)]
        R.ref_image_decode.restype = C.c_int
        R.ref_image_decode.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_uint8), C.c_int, C.POINTER(C.c_int),
                                       C.POINTER(C.c_int), C.POINTER(C.c_int)]
        R.ref_jpeg_encode.restype = C.c_int
        R.ref_jpeg_encode.argtypes = [C.POINTER(C.c_uint8), C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_uint8),
                                      C.c_int]
        _ref = R
    return _ref


def fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def uptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


class OracleScene:
    """The oracle's BVH2 scene over a packed scene view (pt_scene_view)."""

    def __init__(self, view, brute_force: bool = False):
        self._h = C.c_void_p(lib().or_scene_create(C.byref(view), 1 if brute_force else 0))

    def __del__(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().or_scene_destroy(self._h)
            self._h = C.c_void_p(0)

    def render(self, params, rgba: np.ndarray | None = None, sum64: np.ndarray | None = None, rows=None, threads: int = 0):
        """Render params.samples samples from params.sample_index into rgba (H, W, 4) float32."""
        W, H = params.width, params.height
        if rgba is None:
            rgba = np.zeros((H, W, 4), np.float32)
        r0, r1 = rows if rows is not None else (0, H)
        st = OrStats()
        p64 = sum64.ctypes.data_as(C.POINTER(C.c_double)) if sum64 is not None else None
        rc = lib().or_render(self._h, C.byref(params), r0, r1, fptr(rgba), p64, C.byref(st), threads)
        if rc != 0:
            raise RuntimeError("oracle render failed")
        return rgba, st

    def texture_sample(self, index: int, u: float, v: float) -> np.ndarray:
        out = np.zeros(4, np.float32)
        lib().or_texture_sample(self._h, index, u, v, fptr(out))
        return out

    def path_signature(self, params, px: int, py: int, sample_index: int, cap: int = 64):
        out = (C.c_uint64 * cap)()
        n = lib().or_path_signature(self._h, C.byref(params), px, py, sample_index, out, cap)
        return list(out[:n])

    def intersect(self, o, d, tmin=0.0, tmax=float("inf")):
        o = (C.c_float * 3)(*o)
        d = (C.c_float * 3)(*d)
        t, b1, b2 = C.c_float(), C.c_float(), C.c_float()
        inst, prim = C.c_uint32(), C.c_uint32()
        hit = lib().or_intersect(self._h, o, d, tmin, tmax, C.byref(t), C.byref(b1), C.byref(b2), C.byref(inst),
                                 C.byref(prim))
        if not hit:
            return None
        return t.value, b1.value, b2.value, inst.value, prim.value


class OraclePacked:
    """The oracle's packing of a raw scene (its own restatement of SceneBuffer + TableLightSampler)."""

    def __init__(self, raw_struct):
        from pt_gb300 import abi
        self._h = C.c_void_p(lib().or_pack(C.byref(raw_struct)))
        self.view = abi.SceneView()
        lib().or_packed_view(self._h, C.byref(self.view))

    def __del__(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().or_packed_free(self._h)
            self._h = C.c_void_p(0)


def meansq(reference: np.ndarray, image: np.ndarray) -> float:
    ref_ = np.ascontiguousarray(reference, np.float32)
    img = np.ascontiguousarray(image, np.float32)
    H, W = img.shape[:2]
    return lib().or_meansq(fptr(ref_), fptr(img), W, H)


def meansq64(reference_mean: np.ndarray, image: np.ndarray) -> float:
    ref_ = np.ascontiguousarray(reference_mean, np.float64)
    img = np.ascontiguousarray(image, np.float32)
    H, W = img.shape[:2]
    return lib().or_meansq64(ref_.ctypes.data_as(C.POINTER(C.c_double)), fptr(img), W, H)
