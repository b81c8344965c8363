"""Benchmark of the headless path-tracing hot path (one JSON line on rank 0).

Workload (one "step"): the mid-size scene — ~260k instanced triangles in 200
instances of 6 seeded meshes, 32 emissive triangles, thin lens — rendered at
1024x1024 with 128 samples per pixel and at most 8 bounces, FP32 running-mean
accumulation.  Synthetic, seeded scene data (pt_gb300.scenes.mid_scene).

  value   Mpath-segs/s of the device render with the scene and image resident
          in HBM: path segments (primary + extension rays, each with its
          shading and NEE shadow ray) / device time (CUDA events on the render
          stream, which joins the sub-wave streams), summed over the timed
          steps.  L2 is flushed (512 MiB write) between steps, outside the
          event pairs.  The renders run as the library runs them by default
          (two sub-waves in flight); the per-stage times of the roofline come
          from a second pass of the same steps on one stream.
  e2e     the same metric through the C ABI with host buffers: each step
          uploads the packed scene from pinned host memory, builds the BVH,
          renders and reads the image back to host memory.
  roofline  algorithmic bytes per segment (B_seg, fixed per scene from the
          oracle's BVH2 visit counts) x segments / device time, against the
          measured HBM copy bandwidth.
  cpu_baseline  the CPU oracle (the C++ restatement of the reference's shader
          math, OpenMP over pixels) on a bounded sample of the same workload.
  time_to_mse  wall time (synchronised, same scene and image size) for plain
          GPU accumulation and for the denoised pipeline (render + first-hit
          features + U-Net) to reach MSE <= 1e-3 against a 4096-spp image
          accumulated in FP64 on the GPU; `speedup` = plain / denoised.

--impl reference runs the reference's CPU implementation of the path on the
host cores: the reference's Vulkan tracer cannot run on this machine, so this
arm times the oracle port with all host threads.

Multi-GPU (torchrun): replicas with disjoint sample ranges (rank r renders
samples [r*S, (r+1)*S)), weak scaling, no data-path collective.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WIDTH, HEIGHT, SPP, BOUNCES = 1024, 1024, 128, 8
WORKLOAD = "mid scene: 1024x1024, 128 spp, max 8 bounces, ~260k tris / 200 instances / 6 meshes, 32 emitters, thin lens"

# Algorithmic bytes per path segment of the mid scene:
#   B_seg = 128 (path state r/w: the reference's 16-u32 queue item each way)
#         + 332 (hit fetch: InstanceData 128 + PbrMaterial 96 + 3 indices 12 + 3 vertices 96)
#         + p_nee * (40 + 24 + 128 + 96 + 96) (light bin, emitter bin, instance, 3 vertices, material)
#         + (N_node * 64 + N_tri * 36) * (1 + p_nee)
# with N_node, N_tri the mean interior-node visits and triangle tests per ray
# of the oracle's binned-SAH BVH2 over the first sample of the image, and
# p_nee the shadow rays per segment (measured by tests/test_bseg.py, which
# checks these constants against the oracle).
MSE_TARGET = 1e-3
REF_SPP = 4096
DENOISE_SPP = (1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64)

BSEG = {"mid": {"n_node": 27.2106, "n_tri": 9.0453, "p_nee": 0.2336},
        "small": {"n_node": 13.7945, "n_tri": 6.0748, "p_nee": 0.5218},
        "heavy": {"n_node": 70.6501, "n_tri": 24.7050, "p_nee": 0.3352}}


def bseg_bytes(m: dict) -> float | None:
    if m["n_node"] is None:
        return None
    p = m["p_nee"]
    return 128 + 332 + p * (40 + 24 + 128 + 96 + 96) + (m["n_node"] * 64 + m["n_tri"] * 36) * (1 + p)


def extend_bytes(m: dict) -> float:
    """Algorithmic bytes of one closest-hit ray in k_wf_extend (the dominant
    kernel): the traversal term of B_seg for one ray, N_node * 64 + N_tri * 36,
    plus the ray it reads (origin + direction, 32 B), the queue entry (4 B)
    and the hit it writes (t, barycentrics, instance 16 B + primitive 4 B)."""
    return m["n_node"] * 64 + m["n_tri"] * 36 + 32 + 4 + 20


class ClockSampler:
    """Samples nvidia-smi clocks every 200 ms while running."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", "--query-gpu=" + ",".join(self.FIELDS), "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == len(self.FIELDS):
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[0]) for r in self.rows if num(r[0]) is not None]
        mx = [num(r[1]) for r in self.rows if num(r[1]) is not None]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for name, v in zip(names, r[4:8]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def make_scene(workdir: Path):
    import pt_gb300 as P
    from pt_gb300 import scenes
    path = scenes.mid_scene(workdir / "mid", seed=1)
    hs = P.HostScene.load(path)
    return hs


def oracle_scene(workdir: Path):
    """The same mid scene, read and packed by the oracle alone (its own .scn +
    glTF reader and packer): nothing here loads libptgpu.so.  Returns the
    oracle scene, the packed scene (kept alive with it) and a params factory."""
    import oracle
    from oracle import scn_reader
    from pt_gb300 import abi, scenes
    raw, cam = scn_reader.read_scn(scenes.mid_scene(workdir / "mid", seed=1))
    rs, keep = scn_reader.raw_struct(raw)
    packed = oracle.OraclePacked(rs)
    osc = oracle.OracleScene(packed.view)
    cd = scn_reader.camera_desc(cam)

    def params(samples, first):
        p = abi.RenderParams()
        oracle.lib().or_camera_params(cd, WIDTH, HEIGHT, p)
        p.sample_index, p.samples, p.max_bounces, p.rr_start = first, samples, BOUNCES, 1
        return p

    return osc, (packed, keep), params


def cpu_baseline(osc, params_fn, seconds_target: float = 15.0) -> dict:
    """Oracle port on all host threads over a bounded sample of the workload:
    whole frames of consecutive samples (0, 1, 2, ...) until about
    seconds_target of wall time has been spent.  params_fn(samples, first)."""
    threads = os.cpu_count() or 1
    segs, dt, n = 0, 0.0, 0
    while dt < seconds_target:
        t0 = time.perf_counter()
        _, st = osc.render(params_fn(1, n), threads=threads)
        dt += time.perf_counter() - t0
        segs += st.segments
        n += 1
    return {"value": segs / dt / 1e6, "unit": "Mpath-segs/s", "cores": threads, "kind": "port",
            "sample": f"mid scene {WIDTH}x{HEIGHT}, samples 0-{n - 1} of {SPP} ({segs} segments, {dt:.1f} s)",
            "segments": int(segs), "seconds": dt}


def shared_config(world: int) -> dict:
    """The workload, identical in both arms' lines."""
    return {"workload": WORKLOAD, "image": f"{WIDTH}x{HEIGHT}", "spp": SPP, "max_bounces": BOUNCES,
            "l2": "GPU arm: flushed between steps (512 MiB write, outside the event pairs); CPU arm: n/a",
            "parallelism": f"replicas x{world} (disjoint sample ranges)"}


def run_reference(args) -> None:
    """The reference's CPU implementation of the path on the host cores: its
    Vulkan tracer cannot run on this machine (no graphics stack), so the
    oracle port is timed, each step a bounded sample (whole frames of
    consecutive samples for about --ref-seconds).  Scene read and packed by
    the oracle alone; libptgpu.so is never loaded."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    with tempfile.TemporaryDirectory() as td:
        osc, keep, params = oracle_scene(Path(td))
        for _ in range(args.warmup):
            cpu_baseline(osc, params, seconds_target=1.0)
        runs = [cpu_baseline(osc, params, seconds_target=float(args.ref_seconds)) for _ in range(args.steps)]
        v = statistics.median(r["value"] for r in runs)
        line = {"metric": METRIC, "value": v, "unit": "Mpath-segs/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000.0 * statistics.median(r["seconds"] for r in runs),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "impl": "reference", "config": shared_config(world),
                "cpu_baseline": {"value": v, "unit": "Mpath-segs/s", "cores": runs[0]["cores"], "kind": "port",
                                 "sample": runs[0]["sample"] + " per step; the reference's Vulkan tracer is unavailable "
                                                               "on this box (no graphics stack), so its CPU restatement "
                                                               "(the oracle) is timed"},
                "e2e": {"value": v, "unit": "Mpath-segs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "native_libraries": repo_libraries()}
        print(json.dumps(line), flush=True)


METRIC = "time to MSE≤1e-3 vs FP64 ref: denoised vs plain (1 GB300); Mpath-segs/s"


def repo_libraries() -> list:
    """Shared objects of this repository mapped into this process (from
    /proc/self/maps), relative to the repository root."""
    found = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 6 and parts[-1].endswith(".so") and parts[-1].startswith(str(ROOT) + os.sep):
                    found.add(os.path.relpath(parts[-1], ROOT))
    except OSError:
        pass
    return sorted(found)


def pinned_view(view):
    """Copy every array of a packed scene view into pinned host memory (torch)."""
    import ctypes as C
    import numpy as np
    import torch
    from pt_gb300 import abi, view_arrays
    arrs = view_arrays(view)
    keep = []

    def pin(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        keep.append(t)
        return t.data_ptr()

    v = abi.SceneView()
    v.vertices = C.cast(pin(arrs["vertices"]), C.POINTER(C.c_float))
    v.vertex_count = view.vertex_count
    v.indices = C.cast(pin(arrs["indices"]), C.POINTER(C.c_uint32))
    v.index_count = view.index_count
    v.meshes = C.cast(pin(arrs["meshes"]), C.POINTER(abi.MeshRange))
    v.mesh_count = view.mesh_count
    v.instances = C.cast(pin(arrs["instances"]), C.POINTER(abi.InstanceData))
    v.instance_mesh = C.cast(pin(arrs["instance_mesh"]), C.POINTER(C.c_uint32))
    v.instance_world_to_object = C.cast(pin(arrs["w2o"]), C.POINTER(C.c_float))
    v.instance_opaque = C.cast(pin(arrs["opaque"]), C.POINTER(C.c_uint8))
    v.instance_count = view.instance_count
    v.materials = C.cast(pin(arrs["materials"]), C.POINTER(abi.Material))
    v.material_count = view.material_count
    v.light_words = C.cast(pin(arrs["light"]), C.POINTER(C.c_uint32))
    v.light_word_count = view.light_word_count
    v.light_count = view.light_count
    for k in range(3):
        v.environment_colour[k] = view.environment_colour[k]
    nbytes = sum(a.nbytes for a in arrs.values() if hasattr(a, "nbytes"))
    return v, keep, nbytes


def meansq(a, ref) -> float:
    """util/meansq/meansq.cpp:34-43 over RGB: sum of squared differences / (n - 1)."""
    import numpy as np

    d = a[..., :3].astype(np.float64) - ref[..., :3]
    return float(np.sum(d * d) / (d.size - 1))


def time_to_mse(ctx, hs, kernel: int, ref_spp: int, curve: bool = True) -> dict:
    """Wall time (render + read of the converged-enough image, synchronised)
    for plain accumulation and for the denoised pipeline to reach
    MSE <= MSE_TARGET against an FP64-accumulated reference of ref_spp samples."""
    import math
    import numpy as np
    from pt_gb300 import abi
    from pt_gb300.denoise import WEIGHTS_DIR, UNet, load_params

    def params(n, mode=abi.PT_ACCUM_FP32):
        return hs.render_params(WIDTH, HEIGHT, n, BOUNCES, accum_mode=mode, kernel=kernel)

    t0 = time.perf_counter()
    ctx.render(params(ref_spp, abi.PT_ACCUM_FP32_FP64), stats=False)
    ref = ctx.read_image(fp64=True)
    ref_s = time.perf_counter() - t0
    ref32 = np.ascontiguousarray(ref.astype(np.float32))

    def plain(n):
        ctx.synchronize()
        t = time.perf_counter()
        ctx.render(params(n), stats=False)
        ctx.synchronize()
        t = time.perf_counter() - t
        return ctx.mse(ref32), t

    plain(8)  # warm-up
    m16, _ = plain(16)
    n = max(1, int(math.ceil(16 * m16 / MSE_TARGET)))
    m, t = plain(n)
    while m > MSE_TARGET:
        n = int(n * 1.08) + 1
        m, t = plain(n)
    while n > 1:
        k = n - max(1, n // 25)
        mk, tk = plain(k)
        if mk > MSE_TARGET:
            break
        n, m, t = k, mk, tk
    out = {"threshold": MSE_TARGET, "metric": "meansq over RGB (meansq.cpp)",
           "reference": {"spp": ref_spp, "accumulation": "fp64 on the GPU", "seconds": round(ref_s, 3)},
           "plain": {"spp": n, "seconds": t, "mse": m}}
    wfile = WEIGHTS_DIR / "unet.bin"
    if not wfile.exists():
        out["denoised"] = None
        out["denoised_unavailable"] = "no trained weights (run python -m pt_gb300.train_denoiser)"
        return out
    unet = UNet(1, HEIGHT, WIDTH)
    unet.set_params(load_params(wfile))

    def denoised(s):
        p = params(s)
        ctx.synchronize()
        t = time.perf_counter()
        ctx.render_denoised(unet, p)
        ctx.synchronize()
        t = time.perf_counter() - t
        return meansq(ctx.read_denoised(), ref), t

    denoised(4)  # warm-up
    points = {}
    best = None
    for s in DENOISE_SPP:
        m, t = denoised(s)
        points[s] = {"mse": m, "seconds": t, "plain_mse": plain(s)[0] if curve else None}
        if m <= MSE_TARGET:
            best = {"spp": s, "seconds": t, "mse": m}
            break
    out["denoised"] = best
    if curve:
        out["denoised_curve"] = points
    out["speedup"] = (out["plain"]["seconds"] / best["seconds"]) if best else None
    unet.close()
    return out


def time_to_mse_seeds(device_index: int, kernel: int, ref_spp: int, seeds=(2, 3, 4)) -> dict:
    """time_to_mse on mid scenes of other seeds (held out: the denoiser's
    training scenes come from pt_gb300.trainset, not from these)."""
    import pt_gb300 as P
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for s in seeds:
            from pt_gb300 import scenes
            hs = P.HostScene.load(scenes.mid_scene(Path(td) / f"mid{s}", seed=s))
            c = P.Context(device_index)
            c.upload(hs.pack())
            c.build_accel()
            r = time_to_mse(c, hs, kernel, ref_spp, curve=False)
            out[str(s)] = {"plain_spp": r["plain"]["spp"], "plain_s": r["plain"]["seconds"],
                           "denoised_spp": (r["denoised"] or {}).get("spp"),
                           "denoised_s": (r["denoised"] or {}).get("seconds"), "speedup": r.get("speedup")}
            c.close()
    sp = [v["speedup"] for v in out.values() if v["speedup"]]
    return {"seeds": out, "speedup_min": min(sp) if sp else None,
            "speedup_median": statistics.median(sp) if sp else None}


HEAVY = {"width": 1920, "height": 1080, "bounces": 12, "rr_start": 4, "ref_spp": 16384}
HEAVY_DENOISE_SPP = (4, 8, 16, 32, 64, 96, 128, 192, 256, 384, 512, 768, 1024)


def time_to_mse_heavy(device_index: int, ref_spp: int = HEAVY["ref_spp"]) -> dict:
    """Time to MSE <= 1e-3 on the heavy configuration: ~2M unique triangles
    in 64 BLASes, 10,000 instances, 256 emitters, 1920x1080, 12 bounces,
    Russian roulette from segment 4, against a `ref_spp`-sample image
    accumulated in FP64 on the GPU.

    plain     the smallest spp whose running mean reaches the threshold,
              found by rendering progressively (chunks sized from the 1/spp
              decay of the error, down to 8 spp; untimed), then timed as one
              uninterrupted render of that many samples;
    denoised  the first spp of HEAVY_DENOISE_SPP whose denoised image
              reaches it, then bisected between that rung and the one
              below; timed as render (with features and the half-sample
              snapshot) + network, synchronised."""
    import math
    import numpy as np
    import pt_gb300 as P
    from pt_gb300 import abi, scenes
    from pt_gb300.denoise import WEIGHTS_DIR, UNet, load_params

    W, H, B, RR = HEAVY["width"], HEAVY["height"], HEAVY["bounces"], HEAVY["rr_start"]
    raw, cam = scenes.heavy_scene()
    hs = P.HostScene.from_raw(raw, cam)
    ctx = P.Context(device_index)
    ctx.upload(hs.pack())
    ctx.build_accel()

    def params(n, first=0, mode=abi.PT_ACCUM_FP32):
        return hs.render_params(W, H, n, B, sample_index=first, accum_mode=mode, rr_start=RR)

    t0 = time.perf_counter()
    st = ctx.render(params(ref_spp, mode=abi.PT_ACCUM_FP32_FP64))
    ref = ctx.read_image(fp64=True)
    ref_s = time.perf_counter() - t0
    ref32 = np.ascontiguousarray(ref.astype(np.float32))
    out = {"threshold": MSE_TARGET, "metric": "meansq over RGB (meansq.cpp)",
           "config": f"heavy scene {W}x{H}, {B} bounces, Russian roulette from segment {RR}",
           "reference": {"spp": ref_spp, "accumulation": "fp64 on the GPU", "seconds": round(ref_s, 3),
                         "mpath_segs_s": st.segments / st.milliseconds / 1e3}}

    # plain: progressive search (untimed), then one timed render.  The error
    # times spp still falls between 32 and a few hundred spp here (early
    # fireflies), so a 1/spp projection overshoots: each step covers half the
    # projected distance (at least 8 spp), which ends within a few spp of the
    # first sample count that reaches the threshold.
    n, m = 32, None
    ctx.render(params(32), stats=False)
    m = ctx.mse(ref32)
    trail = [(n, m)]
    while m > MSE_TARGET:
        proj = n * m / MSE_TARGET
        step = int(min(512, max(8, round((proj - n) * 0.5))))
        ctx.render(params(step, first=n), stats=False)
        n += step
        m = ctx.mse(ref32)
        trail.append((n, m))
    ctx.synchronize()
    t = time.perf_counter()
    ctx.render(params(n), stats=False)
    ctx.synchronize()
    plain_s = time.perf_counter() - t
    m_check = ctx.mse(ref32)
    out["plain"] = {"spp": n, "seconds": plain_s, "mse": m_check, "previous_step": trail[-2] if len(trail) > 1 else None}

    wfile = WEIGHTS_DIR / "unet.bin"
    if not wfile.exists():
        out["denoised"] = None
        ctx.close()
        return out
    unet = UNet(1, H, W)
    unet.set_params(load_params(wfile))

    def denoised(s):
        p = params(s)
        ctx.synchronize()
        tt = time.perf_counter()
        ctx.render_denoised(unet, p)
        ctx.synchronize()
        tt = time.perf_counter() - tt
        return meansq(ctx.read_denoised(), ref), tt, ctx.mse(ref32)

    denoised(4)  # warm-up
    curve, best, below = {}, None, None
    for s in HEAVY_DENOISE_SPP:
        if s >= n:
            break
        md, td, mp = denoised(s)
        curve[s] = {"mse": md, "seconds": td, "plain_mse": mp}
        if md <= MSE_TARGET:
            best = {"spp": s, "seconds": td, "mse": md}
            break
        below = s
    if best is not None and below is not None:
        lo, hi = below, best["spp"]
        while hi - lo > max(2, lo // 16):
            mid_s = (lo + hi) // 2
            md, td, mp = denoised(mid_s)
            curve[mid_s] = {"mse": md, "seconds": td, "plain_mse": mp}
            if md <= MSE_TARGET:
                hi, best = mid_s, {"spp": mid_s, "seconds": td, "mse": md}
            else:
                lo = mid_s
    out["denoised"] = best
    out["denoised_curve"] = dict(sorted(curve.items()))
    out["speedup"] = plain_s / best["seconds"] if best else None
    if best is None:
        below_plain = [s for s in curve if s < n]
        out["denoised_shortfall"] = (f"the denoised image did not reach MSE {MSE_TARGET} at any tried spp below "
                                     f"plain's {n}; lowest denoised MSE "
                                     f"{min(v['mse'] for v in curve.values()):.4g}" if below_plain else None)
    unet.close()
    ctx.close()
    return out


CONFIG_WORKLOADS = {
    "small": "small scene: 256x256, 16 spp, max 8 bounces, 8 icospheres + ground + lamp (~10k instanced tris), pinhole",
    "heavy": "heavy scene: 1920x1080, 256 spp, max 12 bounces, Russian roulette from segment 4, ~2M unique tris in "
             "64 BLASes, 10,000 instances, 256 emitters"}


def config_leg(device_index: int, name: str, steps: int, cpu_seconds: float, no_cpu: bool) -> dict:
    """Throughput of one more benchmark configuration, measured like the main
    line: device time of `steps` renders (L2 flushed between them, stage
    events for the dominant kernel's roofline), and the oracle on the host
    cores over a bounded sample of the same render.

      small  256x256, 16 spp, 8 bounces: 8 icospheres + ground + lamp (~10k tris)
      heavy  1920x1080, 256 spp, 12 bounces, Russian roulette from segment 4:
             ~2M unique tris in 64 BLASes, 10,000 instances, 256 emitters"""
    import numpy as np
    import torch
    import oracle
    import pt_gb300 as P
    from oracle import scn_reader
    from pt_gb300 import abi, scenes

    if name == "small":
        td = tempfile.TemporaryDirectory()
        path = scenes.small_scene(Path(td.name) / "small", seed=0)
        hs = P.HostScene.load(path)
        raw_o, cam_o = scn_reader.read_scn(path)
        W, H, S, B, RR = 256, 256, 16, 8, 1
    else:
        td = None
        raw_o, cam_o = scenes.heavy_scene()
        hs = P.HostScene.from_raw(raw_o, cam_o)
        cam_o = {"position": cam_o["position"], "lookdir": cam_o["lookdir"], "up": (0.0, 1.0, 0.0),
                 "fov_degrees": cam_o["fov_degrees"], "near_plane": 0.1, "far_plane": 1000.0, "focus_dist": 0.0,
                 "lens_radius": 0.0, "exposure": 1.0}
        W, H, S, B, RR = 1920, 1080, 256, 12, 4
    ctx = P.Context(device_index)
    ctx.upload(hs.pack())
    info = ctx.build_accel()
    p = hs.render_params(W, H, S, B, rr_start=RR)
    st = ctx.render(p)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{device_index}")
    ms, stage, launches = [], [0.0] * 6, 0
    for _ in range(steps):  # the library's default streams
        flush.zero_()
        torch.cuda.synchronize()
        ms.append(ctx.render(p).milliseconds)
    p.flags = abi.PT_RENDER_TIME_STAGES
    for _ in range(steps):  # the same renders on one stream, stage by stage
        flush.zero_()
        torch.cuda.synchronize()
        s = ctx.render(p)
        stage = [a + b for a, b in zip(stage, s.stage_ms)]
        launches += s.stage_launches
    t = sum(ms) / 1000.0
    value = st.segments * steps / t / 1e6
    peaks = measured_peaks()
    ext_b = extend_bytes(BSEG[name])
    ext_s = stage[1] / 1000.0
    out = {"workload": CONFIG_WORKLOADS[name], "image": f"{W}x{H}", "spp": S, "max_bounces": B, "rr_start": RR, "value": value, "unit": "Mpath-segs/s",
           "ms_per_step": 1000.0 * t / steps, "steps": steps, "segments_per_step": int(st.segments),
           "accel_build_ms": info.build_ms,
           "roofline": {"bound": "hbm", "kernel": "k_wf_extend", "bytes_per_ray": ext_b,
                        "achieved": ext_b * st.segments * steps / ext_s / 1e9 if ext_s > 0 else None,
                        "peak": peaks["hbm_gbs"], "unit": "GB/s",
                        "frac": ext_b * st.segments * steps / ext_s / 1e9 / peaks["hbm_gbs"] if ext_s > 0 else None,
                        "avg_launch_ms": stage[1] / max(1, launches),
                        "stage_ms_per_step": {k: v / steps for k, v in zip(abi.STAGES, stage)},
                        "step": {"bytes_per_segment": bseg_bytes(BSEG[name]),
                                 "frac": bseg_bytes(BSEG[name]) * st.segments / (t / steps) / 1e9 / peaks["hbm_gbs"]}}}
    if not no_cpu:
        rs, keep = scn_reader.raw_struct(raw_o)
        packed = oracle.OraclePacked(rs)
        osc = oracle.OracleScene(packed.view)
        cd = scn_reader.camera_desc(cam_o)

        def params(samples, first):
            q = abi.RenderParams()
            oracle.lib().or_camera_params(cd, W, H, q)
            q.sample_index, q.samples, q.max_bounces, q.rr_start = first, samples, B, RR
            return q

        threads = os.cpu_count() or 1
        segs, dt, n = 0, 0.0, 0
        while n < S and (dt < cpu_seconds or n == 0):
            t0 = time.perf_counter()
            _, ost = osc.render(params(1, n), threads=threads)
            dt += time.perf_counter() - t0
            segs += ost.segments
            n += 1
        out["cpu_baseline"] = {"value": segs / dt / 1e6, "unit": "Mpath-segs/s", "cores": threads, "kind": "port",
                               "sample": f"{name} {W}x{H}, samples 0-{n - 1} of {S} ({segs} segments, {dt:.1f} s)"
                                         + (" = the whole render" if n == S else "")}
        del osc, packed, keep
    ctx.close()
    if td is not None:
        td.cleanup()
    return out


def batch_bench(device_index: int, jobs: int = 64, side=(128, 1024), spp=(4, 256), tris=(1000, 500000)) -> dict:
    """The batch workload (scenes.batch_workload: `jobs` jobs, own scene each,
    square side, samples and unique triangles log-uniform in the given
    ranges, 8 bounces) rendered by pt_render_batch (tuned, CUDA graph) and,
    for comparison, job after job with pt_render (wavefront).  The tuner's
    trials and the graph capture run in a first, untimed call; the timed
    batch is the graph launch of a second call (device time)."""
    import numpy as np
    import pt_gb300 as P
    from pt_gb300 import scenes

    spec = scenes.batch_workload(jobs=jobs, side=side, spp=spp, tris=tris)
    ctx = P.Context(device_index)
    keep, js = [], []
    for j in spec:
        raw, cam = scenes.batch_scene(j["seed"], j["tris"])
        hs = P.HostScene.from_raw(raw, cam)
        v = hs.pack()
        c = P.Context(device_index)
        c.upload(v)
        c.build_accel()
        keep.append((hs, v))
        js.append((c, hs.render_params(j["side"], j["side"], j["spp"], j["max_bounces"])))
    first = ctx.render_batch(js)
    st = ctx.render_batch(js)
    done = ctx.batch_job_times()
    seq_ms, seq_segs, seq_done = 0.0, 0, []
    for c, p in js:
        s1 = c.render(p)
        seq_ms += s1.milliseconds
        seq_segs += s1.segments
        seq_done.append(seq_ms)  # job after job in submission order: each job's latency
    out = {"jobs": jobs, "side": list(side), "spp": list(spp), "tris": list(tris),
           "paths": int(st.paths), "segments": int(st.segments),
           "batch_ms": st.milliseconds, "batch_mseg_s": st.segments / st.milliseconds / 1e3,
           "sequential_ms": seq_ms, "sequential_mseg_s": seq_segs / seq_ms / 1e3,
           "speedup_vs_sequential": seq_ms / st.milliseconds,
           "tune_ms": first.tune_milliseconds, "capture_ms": first.build_milliseconds, "graph_reused": int(st.graph_reused),
           "waves": st.waves, "graph_launches": st.kernel_launches, "wave_capacity": st.wave_capacity,
           "mega_jobs": st.mega_jobs, "mega_threshold": int(st.mega_threshold), "tile_w": st.tile_w,
           "job_latency_ms": {"batch_p50": float(np.percentile(done, 50)), "batch_p99": float(np.percentile(done, 99)),
                              "sequential_p50": float(np.percentile(seq_done, 50)),
                              "sequential_p99": float(np.percentile(seq_done, 99)),
                              "note": "time from the start until each job's image is final; sequential = one pt_render "
                                      "after another in submission order"}}
    for c, _ in js:
        c.close()
    ctx.close()
    return out


def run_denoise_profile(args) -> None:
    """The denoised pipeline alone (mid scene, --denoise-profile spp), three
    times after a warm-up: the command profiled for the denoiser's launch list."""
    import pt_gb300 as P
    from pt_gb300.denoise import WEIGHTS_DIR, UNet, init_params, load_params

    td = tempfile.TemporaryDirectory()
    hs = make_scene(Path(td.name))
    ctx = P.Context(0)
    ctx.upload(hs.pack())
    ctx.build_accel()
    unet = UNet(1, HEIGHT, WIDTH)
    wfile = WEIGHTS_DIR / "unet.bin"
    unet.set_params(load_params(wfile) if wfile.exists() else init_params(0))
    s = args.denoise_profile
    p = hs.render_params(WIDTH, HEIGHT, s, BOUNCES, kernel=args.kernel)
    times = []
    for i in range(4):
        ctx.synchronize()
        t = time.perf_counter()
        ctx.render_denoised(unet, p)
        ctx.synchronize()
        times.append(time.perf_counter() - t)
    # the same pipeline stage by stage (synchronised after each)
    stages = {}

    def stage(name, fn):
        ctx.synchronize()
        t0 = time.perf_counter()
        fn()
        ctx.synchronize()
        stages[name] = stages.get(name, 0.0) + time.perf_counter() - t0

    for i in range(3):
        stage("render_with_features_and_snapshot", lambda: ctx.render_noisy(hs.render_params(WIDTH, HEIGHT, s, BOUNCES,
                                                                                          kernel=args.kernel)))
        stage("network", lambda: ctx.denoise(unet, s))
    one = hs.render_params(WIDTH, HEIGHT, s, BOUNCES, kernel=args.kernel)
    stage("plain_render_same_spp", lambda: ctx.render(one, stats=False))
    stages = {k: v / 3 if k != "plain_render_same_spp" else v for k, v in stages.items()}
    print(json.dumps({"denoise_profile_spp": s, "seconds": times[1:], "stages_s": stages}))
    unet.close()
    ctx.close()
    td.cleanup()


def run_ours(args) -> None:
    import numpy as np
    import torch
    import pt_gb300 as P
    from pt_gb300 import abi

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = world > 1
    if dist:
        import torch.distributed as tdist
        tdist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    device_index = local

    td = tempfile.TemporaryDirectory()
    hs = make_scene(Path(td.name))
    view = hs.pack()
    pview, keep, scene_bytes = pinned_view(view)
    ctx = P.Context(device_index)
    ctx.upload(view)
    info = ctx.build_accel()
    first = rank * SPP

    def params(n=SPP, start=first, flags=0):
        p = hs.render_params(WIDTH, HEIGHT, n, BOUNCES, sample_index=start, kernel=args.kernel)
        p.flags = flags
        return p

    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{device_index}")

    def l2_flush():
        flush.zero_()
        torch.cuda.synchronize()

    # warm-up (also gives the deterministic segment count of one step)
    st = None
    for _ in range(max(args.warmup, 1)):
        st = ctx.render(params())
    segs_per_step = st.segments
    launches_per_step = st.kernel_launches

    # ---- device-resident timing: K renders as the library runs them (its
    # default sub-wave streams), then the same K renders on one stream with
    # events between the stages (per-stage times for the roofline; stage
    # events need a single stream)
    dev_ms = []
    stage_ms = [0.0] * 6
    stage_step_ms = []
    stage_launches = 0
    if dist:
        tdist.barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    with ClockSampler(device_index) as clocks:
        for _ in range(args.steps):
            l2_flush()
            s = ctx.render(params())
            if s.segments != segs_per_step:
                raise RuntimeError("segment count changed between identical renders")
            dev_ms.append(s.milliseconds)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        for _ in range(args.steps):
            l2_flush()
            s = ctx.render(params(flags=abi.PT_RENDER_TIME_STAGES))
            if s.segments != segs_per_step:
                raise RuntimeError("segment count changed between identical renders")
            stage_step_ms.append(s.milliseconds)
            stage_ms = [a + b for a, b in zip(stage_ms, s.stage_ms)]
            stage_launches += s.stage_launches
    torch.cuda.synchronize()
    t_dev = sum(dev_ms) / 1000.0
    if dist:
        t = torch.tensor([t_dev], device=f"cuda:{device_index}")
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        t_dev = float(t.item())
    total_segs = segs_per_step * args.steps * world
    value = total_segs / t_dev / 1e6

    # ---- end to end through the C ABI with host buffers
    t_e2e = float("nan")
    if not args.no_e2e:
        img = torch.empty((HEIGHT, WIDTH, 4), dtype=torch.float32).pin_memory()
        e2e_ctx = P.Context(device_index)
        e2e_ctx.upload(pview)
        e2e_ctx.build_accel()
        e2e_ctx.render(params(4))
        e2e_ctx.read_image(out=img.numpy())
        if dist:
            tdist.barrier()
        torch.cuda.synchronize()
        e0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_ctx.upload(pview)
            e2e_ctx.build_accel()
            e2e_ctx.render(params(), stats=False)
            e2e_ctx.read_image(out=img.numpy())
        torch.cuda.synchronize()
        t_e2e = time.perf_counter() - e0
        if dist:
            t = torch.tensor([t_e2e], device=f"cuda:{device_index}")
            tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
            t_e2e = float(t.item())
        e2e_ctx.close()
    e2e_value = total_segs / t_e2e / 1e6

    if rank == 0:
        peaks = measured_peaks()
        peak_src = "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks["source"] == "measured" else "fallback"
        b = bseg_bytes(BSEG["mid"])
        step_achieved = b * segs_per_step / (t_dev / args.steps) / 1e9
        # The dominant kernel is k_wf_extend (closest-hit traversal): its
        # launches are timed by CUDA events recorded between the wavefront's
        # launches on the render stream (PT_RENDER_TIME_STAGES) over the timed
        # steps.  One launch traces the queued rays of one segment of a wave.
        ext_b = extend_bytes(BSEG["mid"])
        ext_s = stage_ms[1] / 1000.0
        ext_launches = max(1, stage_launches)
        rays_per_launch = segs_per_step * args.steps / ext_launches
        ext_achieved = ext_b * segs_per_step * args.steps / ext_s / 1e9 if ext_s > 0 else None
        # DRAM bytes per extend launch: ncu's dram__bytes_read.sum +
        # dram__bytes_write.sum of k_wf_extend per traced ray on a smaller
        # capture of the same scene (profiles/traffic.json), times the rays of
        # an average launch here.
        traffic = None
        tfile = ROOT / "profiles" / "traffic.json"
        if tfile.exists():
            per_ray = json.loads(tfile.read_text()).get("mid_wavefront", {}).get("extend_dram_bytes_per_ray")
            if per_ray:
                traffic = per_ray * rays_per_launch
        roof = {"bound": "hbm", "kernel": "k_wf_extend", "achieved": ext_achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": (ext_achieved / peaks["hbm_gbs"]) if ext_achieved else None, "traffic": traffic,
                "algorithmic_bytes": ext_b * rays_per_launch, "bytes_per_ray": ext_b,
                "launches": stage_launches, "avg_launch_ms": stage_ms[1] / ext_launches, "rays_per_launch": rays_per_launch,
                "peak_source": peak_src,
                "stage_ms_per_step": {k: v / args.steps for k, v in zip(abi.STAGES, stage_ms)},
                "stage_timed_ms_per_step": sum(stage_step_ms) / args.steps,
                "step": {"achieved": step_achieved, "frac": step_achieved / peaks["hbm_gbs"], "bytes_per_segment": b,
                         "note": "whole render step: B_seg x segments / step time"}}
        base = None
        if not args.no_cpu:
            osc, keep_o, oparams = oracle_scene(Path(td.name) / "oracle")
            base = cpu_baseline(osc, oparams, seconds_target=float(args.cpu_seconds))
            del osc, keep_o
        ttm = None
        if not args.no_mse:
            ttm = time_to_mse(ctx, hs, args.kernel, args.ref_spp)
            if not args.no_seeds:
                ttm["held_out_seeds"] = time_to_mse_seeds(device_index, args.kernel, args.ref_spp)
            if not args.no_heavy:
                ttm["heavy"] = time_to_mse_heavy(device_index, args.heavy_ref_spp)
        configs = None
        if not args.no_configs:
            configs = {"small": config_leg(device_index, "small", 5, 5.0, args.no_cpu),
                       "heavy": config_leg(device_index, "heavy", 2, 5.0, args.no_cpu)}
        batches = None
        if not args.no_batch:
            batches = {"uneven_64": batch_bench(device_index),
                       "small_64": batch_bench(device_index, side=(128, 256), spp=(4, 16), tris=(1000, 50000))}
        line = {"metric": METRIC, "value": value, "unit": "Mpath-segs/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000.0 * t_dev / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": shared_config(world),
                "details": {"kernel": {1: "megakernel", 2: "wavefront"}.get(st.kernel_used, str(st.kernel_used)),
                           "wave_streams": "value, e2e and time_to_mse: the library default (PT_WAVE_STREAMS, 2 sub-waves in "
                                           "flight); roofline stage times: a second pass of the same steps on one stream "
                                           "(per-launch stage events need one stream)",
                           "segments_per_step": int(segs_per_step), "accel_build_ms": info.build_ms,
                           "image": f"{WIDTH}x{HEIGHT}", "spp": SPP,
                           "node_visits_per_ray": st.node_visits / max(1, st.segments + st.shadow_rays),
                           "tri_tests_per_ray": st.tri_tests / max(1, st.segments + st.shadow_rays),
                           "shadow_rays_per_segment": st.shadow_rays / max(1, st.segments)},
                "e2e": {"value": e2e_value, "unit": "Mpath-segs/s", "h2d_bytes_per_step": int(scene_bytes),
                        "d2h_bytes_per_step": int(HEIGHT * WIDTH * 16), "ms_per_step": 1000.0 * t_e2e / args.steps,
                        "includes": "scene upload + BVH build + render + image read-back"},
                "gpu_launches": int(launches_per_step * args.steps),
                "roofline": roof, "cpu_baseline": base, "clocks": clocks.summary(), "time_to_mse": ttm, "batch": batches,
                "configs": configs,
                "native_libraries": repo_libraries(),
                "wall_s_timed_region": wall}
        print(json.dumps(line), flush=True)
    ctx.close()
    td.cleanup()
    if dist:
        tdist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--kernel", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU baseline sample of our arm's line")
    ap.add_argument("--ref-seconds", type=float, default=8.0, help="CPU work per step of the reference arm")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-mse", action="store_true", help="skip the time-to-MSE measurement")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-rendering measurement")
    ap.add_argument("--no-configs", action="store_true", help="skip the small and heavy configuration lines")
    ap.add_argument("--ref-spp", type=int, default=REF_SPP)
    ap.add_argument("--no-seeds", action="store_true", help="skip time to MSE on held-out mid-scene seeds")
    ap.add_argument("--no-heavy", action="store_true", help="skip time to MSE on the heavy configuration")
    ap.add_argument("--heavy-ref-spp", type=int, default=HEAVY["ref_spp"])
    ap.add_argument("--heavy-only", action="store_true", help="only the heavy time-to-MSE leg (one JSON line)")
    ap.add_argument("--denoise-profile", type=int, default=0, help="only run the denoised pipeline at this spp (profiling)")
    ap.add_argument("--width", type=int, default=1024, help="smaller images only for profiling captures")
    ap.add_argument("--height", type=int, default=1024)
    ap.add_argument("--spp", type=int, default=128)
    args = ap.parse_args()
    global WIDTH, HEIGHT, SPP
    WIDTH, HEIGHT, SPP = args.width, args.height, args.spp
    if args.warmup < 3:
        args.warmup = 3
    if args.heavy_only:
        print(json.dumps({"time_to_mse_heavy": time_to_mse_heavy(0, args.heavy_ref_spp)}), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    elif args.denoise_profile:
        run_denoise_profile(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
