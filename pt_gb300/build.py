"""Build of the native parts: libptgpu.so (CUDA kernels + C ABI + scene front
end) and the `pt` command-line program, in-tree under pt_gb300/_build/.

Compiles for sm_103a only.  Device code is compiled with -fmad=false so its
float arithmetic follows the reference shaders' expression order without
fused multiply-adds (the CPU oracle is compiled the same way).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = BUILD / "libptgpu.so"
LIB_CHECKED = BUILD / "libptgpu_checked.so" # the same library with bounds-checked kernels (-DPT_CHECKED)
CLI = BUILD / "pt"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr"] + ARCH
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function"]

CU_SOURCES = ["api.cu", "batch.cu", "render_mega.cu", "render_wave.cu", "bvh_build.cu", "post.cu", "noalloc.cu", "features.cu",
              "nn/conv.cu", "nn/conv_rows.cu", "nn/ops.cu", "nn/unet.cu", "nn/api_nn.cu"]
# The denoiser is not on the bit-exact path: let it contract multiply-adds.
NN_FLAGS = [f for f in NVCC_FLAGS if f != "-fmad=false"]
CPP_SOURCES = ["host/scene.cpp", "host/imageio.cpp", "host/png.cpp", "host/jpeg.cpp", "host/assimp_post.cpp"]
HEADERS = list(CSRC.rglob("*.cuh")) + list(CSRC.rglob("*.h")) + list((HERE.parent / "include").glob("*.h"))


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run_parallel(jobs):
    procs = [(name, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for name, cmd in jobs]
    failed = []
    for name, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((name, out))
    if failed:
        msg = "\n".join(f"--- {n}\n{o}" for n, o in failed)
        raise RuntimeError(f"native build failed:\n{msg}")


def build(verbose: bool = False) -> Path:
    """Compile libptgpu.so and the pt CLI if any source changed; return the library path."""
    BUILD.mkdir(parents=True, exist_ok=True)
    jobs, objs = [], []
    for src in CU_SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        objs.append(obj)
        if _stale(obj, [CSRC / src] + HEADERS):
            flags = NN_FLAGS if src.startswith("nn/") else NVCC_FLAGS
            jobs.append((src, [NVCC] + flags + ["-c", str(CSRC / src), "-o", str(obj)]))
    for src in CPP_SOURCES + ["host/main.cpp"]:
        obj = BUILD / (Path(src).stem + ".o")
        if src != "host/main.cpp":
            objs.append(obj)
        if _stale(obj, [CSRC / src] + HEADERS):
            jobs.append((src, ["g++"] + CXX_FLAGS + ["-c", str(CSRC / src), "-o", str(obj)]))
    # the bounds-checked variant: the tracer's translation units again with -DPT_CHECKED
    checked_objs = []
    for src, obj in zip(CU_SOURCES, objs):
        if src.startswith("nn/"):
            checked_objs.append(obj)
            continue
        cobj = BUILD / (Path(src).stem + "_checked.o")
        checked_objs.append(cobj)
        if _stale(cobj, [CSRC / src] + HEADERS):
            jobs.append((src + " (checked)", [NVCC] + NVCC_FLAGS + ["-DPT_CHECKED", "-c", str(CSRC / src), "-o", str(cobj)]))
    checked_objs += objs[len(CU_SOURCES):]
    if jobs:
        if verbose:
            print("building:", ", ".join(n for n, _ in jobs), file=sys.stderr)
        _run_parallel(jobs)
    links = []
    if _stale(LIB, objs):
        links.append(("link libptgpu.so", [NVCC] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs]))
    if _stale(LIB_CHECKED, checked_objs):
        links.append(("link libptgpu_checked.so", [NVCC] + ARCH + ["-shared", "-o", str(LIB_CHECKED)] + [str(o) for o in checked_objs]))
    if links:
        _run_parallel(links)
    main_obj = BUILD / "main.o"
    if _stale(CLI, [main_obj, LIB]):
        _run_parallel([("link pt", ["g++", "-o", str(CLI), str(main_obj), f"-L{BUILD}", "-lptgpu", f"-Wl,-rpath,{BUILD}"])])
    return LIB


def clean() -> None:
    shutil.rmtree(BUILD, ignore_errors=True)


if __name__ == "__main__":
    print(build(verbose=True))
