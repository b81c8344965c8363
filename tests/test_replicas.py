"""Replicas across processes (the multi-GPU path of this library):
disjoint sample ranges per rank, FP64 sums merged with an all-reduce.  Run
on CPU with world size 2 and 3 over gloo; each rank's partial sums come
from the oracle (the GPU renders the same per-sample values
bit for bit, tests/test_gpu_parity.py), so what is tested here is the split,
the merge and the mean."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

import oracle
import pt_gb300 as P
from pt_gb300 import abi, replicas, scenes

TOTAL = 7
W, H = 24, 16


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sample_ranges_cover_and_are_disjoint():
    for total in (0, 1, 5, 128, 129):
        for world in (1, 2, 3, 8):
            got = [replicas.sample_range(total, r, world) for r in range(world)]
            assert got[0][0] == 0
            for (f0, c0), (f1, _) in zip(got, got[1:]):
                assert f0 + c0 == f1
            assert sum(c for _, c in got) == total
            assert max(c for _, c in got) - min(c for _, c in got) <= 1
    with pytest.raises(ValueError):
        replicas.sample_range(4, 2, 2)


def _scene():
    raw, cam = scenes.tiny_raw("two_tris")
    hs = P.HostScene.from_raw(raw, cam)
    return hs, hs.pack()


def _oracle_sums(view, params, first, count):
    s64 = np.zeros((H, W, 4), np.float64)
    if count:
        p = abi.RenderParams.from_buffer_copy(params)
        p.sample_index, p.samples = first, count
        oracle.OracleScene(view, brute_force=True).render(p, sum64=s64)
    return s64


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        hs, view = _scene()
        params = hs.render_params(W, H, TOTAL, 4)
        first, count = replicas.sample_range(TOTAL, rank, world)
        merged = replicas.merge_sums(_oracle_sums(view, params, first, count))
        np.save(os.path.join(out_dir, f"merged_{rank}.npy"), merged)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_gloo_merge_equals_one_process(tmp_path, world):
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
        assert p.exitcode == 0
    hs, view = _scene()
    single = _oracle_sums(view, hs.render_params(W, H, TOTAL, 4), 0, TOTAL)
    for r in range(world):
        merged = np.load(tmp_path / f"merged_{r}.npy")
        assert np.array_equal(merged[..., 3], single[..., 3])  # sample counts exact
        np.testing.assert_allclose(merged[..., :3], single[..., :3], rtol=1e-12, atol=1e-12)
        img = replicas.mean_from_sums(merged)
        np.testing.assert_allclose(img[..., :3], single[..., :3] / TOTAL, rtol=1e-12, atol=1e-12)
