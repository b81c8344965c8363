"""The C ABI: the library loads, exports every entry point the headers
declare, and the ctypes mirror has the C layouts.  No compute calls."""
import ctypes as C
import re
import subprocess
import tempfile
from pathlib import Path

import pytest

from pt_gb300 import abi

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(pt_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_headers_declare_entry_points():
    names = declared_functions()
    assert {"pt_create", "pt_destroy", "pt_upload_scene", "pt_build_accel", "pt_render", "pt_read_image",
            "pt_last_error", "pt_scene_load", "pt_scene_pack"} <= names


def test_library_exports_every_declared_symbol():
    lib = abi.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_checked_library_exports_the_same_symbols():
    """libptgpu_checked.so (bounds-checked kernels) is a drop-in for libptgpu.so."""
    path = abi.LIB_PATH.with_name("libptgpu_checked.so")
    assert path.exists(), path
    lib = C.CDLL(str(path))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    lib.pt_abi_version.restype = C.c_int
    assert lib.pt_abi_version() == abi.ABI_VERSION


def test_ctypes_signatures_cover_declarations():
    assert {n for n, _, _ in abi.SIGNATURES} == declared_functions()


def test_abi_version():
    assert abi.lib().pt_abi_version() == abi.ABI_VERSION == 2


def test_struct_layouts_match_c():
    structs = {"pt_mesh_range": abi.MeshRange, "pt_instance_data": abi.InstanceData, "pt_material": abi.Material,
               "pt_scene_view": abi.SceneView, "pt_render_params": abi.RenderParams, "pt_render_stats": abi.RenderStats,
               "pt_accel_info": abi.AccelInfo, "pt_raw_scene": abi.RawScene, "pt_camera_desc": abi.CameraDesc,
               "pt_texture": abi.Texture, "pt_batch_job": abi.BatchJob, "pt_batch_stats": abi.BatchStats}
    src = '#include <stdio.h>\n#include <stddef.h>\n#include "pt_scene.h"\nint main(void){\n'
    for name in structs:
        src += f'printf("{name} %zu\\n", sizeof({name}));\n'
    src += 'printf("off_view_light %zu\\n", offsetof(pt_scene_view, light_words));\n'
    src += 'printf("off_params_samples %zu\\n", offsetof(pt_render_params, samples));\nreturn 0;}\n'
    with tempfile.TemporaryDirectory() as td:
        (Path(td) / "s.c").write_text(src)
        subprocess.run(["gcc", "-I", str(ROOT / "include"), "-o", f"{td}/s", f"{td}/s.c"], check=True)
        out = subprocess.run([f"{td}/s"], capture_output=True, text=True, check=True).stdout
    sizes = dict(line.split() for line in out.strip().splitlines())
    for name, cls in structs.items():
        assert int(sizes[name]) == C.sizeof(cls), name
    assert int(sizes["off_view_light"]) == abi.SceneView.light_words.offset
    assert int(sizes["off_params_samples"]) == abi.RenderParams.samples.offset
    assert C.sizeof(abi.InstanceData) == 128 and C.sizeof(abi.Material) == 96


def test_create_without_gpu_fails_loudly(has_gpu):
    if has_gpu:
        pytest.skip("a GPU is present")
    h = abi.lib().pt_create(0)
    assert not h
    assert abi.lib().pt_last_error(None)


def test_null_arguments_are_rejected():
    lib = abi.lib()
    assert lib.pt_upload_scene(None, None) == abi.PT_ERR_INVALID
    assert lib.pt_render(None, None, None) == abi.PT_ERR_INVALID
    assert lib.pt_read_image(None, None, 0, 0) == abi.PT_ERR_INVALID
    assert lib.pt_scene_pack(None, None) == abi.PT_ERR_INVALID
    assert not lib.pt_scene_load(None)
