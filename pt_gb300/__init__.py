"""pt_gb300 — GB300-native implementation of pt's headless path-tracing path.

Native library: pt_gb300/_build/libptgpu.so (CUDA kernels for sm_103a, the
C ABI of include/pt_gpu.h and the scene front end of include/pt_scene.h).
"""
from . import abi
from .abi import PtError, NativeLibraryMissing
from .core import Context, HostScene, PathTraceDispatcher, PathTraceParameters, view_arrays

__all__ = ["abi", "PtError", "NativeLibraryMissing", "Context", "HostScene", "PathTraceDispatcher",
           "PathTraceParameters", "view_arrays"]
