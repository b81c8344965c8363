"""pt_gb300 — GB300-native implementation of pt's headless path-tracing path.

Native library: pt_gb300/_build/libptgpu.so (CUDA kernels for sm_103a, the
C ABI of include/pt_gpu.h and the scene front end of include/pt_scene.h).

The submodules load on first use: importing `pt_gb300.abi` (the ctypes
layouts of the C ABI) or `pt_gb300.scenes` (the scene generators) neither
imports the object wrappers of `pt_gb300.core` nor loads the library.
"""
import importlib

_CORE = ("Context", "HostScene", "PathTraceDispatcher", "PathTraceParameters", "view_arrays")
_ABI = ("PtError", "NativeLibraryMissing")

__all__ = ["abi", "PtError", "NativeLibraryMissing", "Context", "HostScene", "PathTraceDispatcher",
           "PathTraceParameters", "view_arrays"]


def __getattr__(name):
    if name in _CORE:
        return getattr(importlib.import_module(".core", __name__), name)
    if name in _ABI:
        return getattr(importlib.import_module(".abi", __name__), name)
    if name == "abi":
        return importlib.import_module(".abi", __name__)
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")
