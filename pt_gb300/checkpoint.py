"""Checkpoint / resume on disk.

Renders.  Progressive accumulation keeps a running mean per pixel whose
update depends only on the sample index (pathtrace.rg.hlsl:62-67), and the
sampler is indexed by the global sample number (pathtrace.rg.hlsl:16), so a
long render cut into chunks of samples and restored between them
(pt_restore_image) gives the image an uninterrupted render gives, bit for
bit.  `render_progressive` renders `total` samples in chunks and after each
chunk writes the running mean, the FP64 sums and the sample count to an
.npz file (written to a temporary name, then renamed, so a crash leaves the
previous checkpoint intact); started again with the same file, it resumes
after the last completed chunk.  A fingerprint of the scene and the render
settings guards against resuming a different render.

Training.  `save_training` / `load_training` store the denoiser's parameters,
both Adam moments, the Adam step count, the training step and the batch
sampler's RNG state, which is everything the next step depends on.
"""
from __future__ import annotations

import hashlib
import os
from pathlib import Path

import numpy as np

from . import abi

RENDER_FORMAT = 1
TRAIN_FORMAT = 1


def _atomic_savez(path: Path, **arrays) -> None:
    path = Path(path)
    tmp = path.with_name(path.name + ".tmp")
    with open(tmp, "wb") as f:
        np.savez(f, **arrays)
        f.flush()
        os.fsync(f.fileno())
    os.replace(tmp, path)


def render_fingerprint(view: abi.SceneView, params: abi.RenderParams) -> str:
    """Hash of the packed scene arrays and of every render setting except
    the sample range, the flags, the accumulation mode and the kernel
    choice (the wavefront and the megakernel give the same samples)."""
    from .core import view_arrays

    h = hashlib.sha256()
    for name, arr in sorted(view_arrays(view).items()):
        h.update(name.encode())
        h.update(np.ascontiguousarray(arr).tobytes())
    p = abi.RenderParams.from_buffer_copy(params)
    p.sample_index, p.samples, p.flags, p.accum_mode, p.kernel = 0, 0, 0, 0, 0
    h.update(bytes(p))
    return h.hexdigest()


def save_render(path, ctx, samples_done: int, fingerprint: str) -> None:
    """Writes the context's running mean, FP64 sums and sample count."""
    from .replicas import read_sums

    _atomic_savez(path, format=np.array(RENDER_FORMAT), rgba=ctx.read_image(), sums64=read_sums(ctx),
                  samples_done=np.array(samples_done, np.int64), fingerprint=np.array(fingerprint))


def load_render(path, ctx, fingerprint: str | None = None) -> int:
    """Restores a checkpoint into `ctx` and returns its sample count.
    Raises ValueError when the file belongs to another scene or setting."""
    with np.load(path, allow_pickle=False) as z:
        if int(z["format"]) != RENDER_FORMAT:
            raise ValueError(f"{path}: checkpoint format {int(z['format'])}, expected {RENDER_FORMAT}")
        if fingerprint is not None and str(z["fingerprint"]) != fingerprint:
            raise ValueError(f"{path}: checkpoint of another scene or render setting")
        done = int(z["samples_done"])
        ctx.restore_image(z["rgba"], done, z["sums64"])
    return done


def render_progressive(ctx, view: abi.SceneView, params: abi.RenderParams, total: int, path, chunk: int = 256,
                       stop_after: int | None = None) -> int:
    """Renders samples [0, total) of `params` into `ctx` with FP64 sums,
    checkpointing to `path` after every `chunk` samples and resuming from it
    when it exists.  `stop_after` ends the call after that many chunks (a
    bounded slice of a long render).  Returns the samples done."""
    if total <= 0 or chunk <= 0:
        raise ValueError("total and chunk must be positive")
    fp = render_fingerprint(view, params)
    path = Path(path)
    done = load_render(path, ctx, fp) if path.exists() else 0
    if done > total:
        raise ValueError(f"{path}: checkpoint holds {done} samples, more than the {total} asked for")
    chunks = 0
    while done < total and (stop_after is None or chunks < stop_after):
        p = abi.RenderParams.from_buffer_copy(params)
        p.sample_index, p.samples = done, min(chunk, total - done)
        p.accum_mode = abi.PT_ACCUM_FP32_FP64
        ctx.render(p, stats=False)
        done += p.samples
        save_render(path, ctx, done, fp)
        chunks += 1
    return done


def save_training(path, net, step: int, rng_state, meta: dict | None = None) -> None:
    """Parameters, Adam moments and step count, the training step and the
    batch sampler's RNG state (a torch.Generator state tensor)."""
    m, v, t = net.adam_state()
    extra = {f"meta_{k}": np.array(val) for k, val in (meta or {}).items()}
    _atomic_savez(path, format=np.array(TRAIN_FORMAT), params=net.params(), adam_m=m, adam_v=v,
                  adam_step=np.array(t, np.int64), step=np.array(step, np.int64),
                  rng_state=np.asarray(rng_state.numpy() if hasattr(rng_state, "numpy") else rng_state, np.uint8),
                  **extra)


def load_training(path, net):
    """Puts parameters and optimizer state back into `net`; returns
    (training step, RNG state as uint8 array, meta dict)."""
    with np.load(path, allow_pickle=False) as z:
        if int(z["format"]) != TRAIN_FORMAT:
            raise ValueError(f"{path}: checkpoint format {int(z['format'])}, expected {TRAIN_FORMAT}")
        net.set_params(z["params"])
        net.set_adam_state(z["adam_m"], z["adam_v"], int(z["adam_step"]))
        meta = {k[5:]: z[k].item() for k in z.files if k.startswith("meta_")}
        return int(z["step"]), z["rng_state"].copy(), meta
