"""Replicas on several GPUs (one process per GPU): disjoint sample ranges.

The sampler's index is the global sample index (pathtrace.rg.hlsl:16), so
rank r of `world` rendering samples [first_r, first_r + count_r) takes
exactly the samples one GPU would take for them; the scene is replicated.
The images merge as FP64 sums (rgb radiance sums + sample count per pixel,
pt_read_image(..., PT_IMAGE_SUMS64)): an element-wise sum over ranks, done
with torch.distributed (gloo through host memory, or NCCL), then one
division.  No collective runs on the rendering path itself.
"""
from __future__ import annotations

import numpy as np

from . import abi
from .core import Context, _check, lib


def sample_range(total: int, rank: int, world: int) -> tuple[int, int]:
    """(first sample, count) of `rank`: `total` samples split into `world`
    contiguous ranges whose sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world or total < 0:
        raise ValueError("bad rank / world / total")
    base, extra = divmod(total, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def read_sums(ctx: Context) -> np.ndarray:
    """The context's FP64 sums [h, w, 4] (needs PT_ACCUM_FP32_FP64 renders)."""
    out = np.empty((ctx.height, ctx.width, 4), np.float64)
    _check(lib().pt_read_image(ctx._h, out.ctypes.data, out.strides[0], abi.PT_IMAGE_SUMS64), ctx._h)
    return out


def render_partial(ctx: Context, params: abi.RenderParams, total: int, rank: int, world: int) -> np.ndarray:
    """Renders this rank's share of `total` samples into cleared FP64 sums
    (PT_RENDER_RESTART) and returns them."""
    first, count = sample_range(total, rank, world)
    p = abi.RenderParams.from_buffer_copy(params)
    if count == 0:
        return np.zeros((p.height, p.width, 4), np.float64)
    p.sample_index, p.samples, p.accum_mode = first, count, abi.PT_ACCUM_FP32_FP64
    p.flags |= abi.PT_RENDER_RESTART
    ctx.render(p, stats=False)
    return read_sums(ctx)


def merge_sums(sums: np.ndarray, group=None) -> np.ndarray:
    """Element-wise sum of every rank's FP64 sums (torch.distributed all_reduce)."""
    import torch
    import torch.distributed as dist

    t = torch.from_numpy(np.ascontiguousarray(sums, np.float64))
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        return t.cpu().numpy()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.numpy()


def mean_from_sums(sums: np.ndarray) -> np.ndarray:
    """RGBA mean image (alpha 1) from merged FP64 sums."""
    cnt = np.where(sums[..., 3:4] > 0, sums[..., 3:4], 1.0)
    out = np.empty_like(sums)
    out[..., :3] = sums[..., :3] / cnt
    out[..., 3] = 1.0
    return out
