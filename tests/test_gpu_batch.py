"""pt_render_batch: many jobs (own scene, camera, size, samples, bounces) in
one launch sequence.  Every job's image must equal rendering that job alone,
bit for bit, whatever the wave packing, the tuner's choice or the graph."""
import ctypes as C

import numpy as np
import pytest

import oracle
import pt_gb300 as P
from pt_gb300 import abi, scenes

pytestmark = pytest.mark.gpu

# (seed, unique triangles, width, height, samples, max bounces)
SPECS = [(11, 2000, 40, 32, 5, 4), (12, 800, 24, 24, 9, 3), (13, 5000, 64, 48, 3, 6), (14, 1500, 16, 16, 12, 2),
         (15, 3000, 56, 40, 7, 8), (16, 1200, 32, 32, 1, 5)]


@pytest.fixture(scope="module")
def batch():
    ctx = P.Context(0)
    keep, jobs = [], []
    for seed, tris, w, h, spp, b in SPECS:
        raw, cam = scenes.batch_scene(seed, tris)
        hs = P.HostScene.from_raw(raw, cam)
        view = hs.pack()
        c = P.Context(0)
        c.upload(view)
        c.build_accel()
        keep.append((hs, view))
        jobs.append((c, hs.render_params(w, h, spp, b)))
    yield ctx, jobs, keep
    for c, _ in jobs:
        c.close()
    ctx.close()


def _single(jobs, kernel=abi.PT_KERNEL_WAVEFRONT):
    out = []
    for c, p in jobs:
        q = abi.RenderParams.from_buffer_copy(p)
        q.kernel = kernel
        c.render(q)
        out.append(c.read_image().copy())
    return out


def _same(a, b):
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("flags", [abi.PT_BATCH_NO_TUNE | abi.PT_BATCH_NO_GRAPH, abi.PT_BATCH_NO_TUNE, 0,
                                   abi.PT_BATCH_NO_TUNE | abi.PT_BATCH_CAPACITY_LOG2(12),
                                   abi.PT_BATCH_CAPACITY_LOG2(13)])
def test_batch_equals_single_renders(batch, flags):
    ctx, jobs, _ = batch
    ref = _single(jobs)
    st = ctx.render_batch(jobs, flags)
    assert st.error_word == 0
    for j in range(len(jobs)):
        assert _same(ctx.read_batch_image(j), ref[j]), j
    assert st.paths == sum(w * h * s for _, _, w, h, s, _ in SPECS)
    if flags & abi.PT_BATCH_CAPACITY_LOG2(31):
        assert st.wave_capacity == 1 << ((flags >> 8) & 31) and st.waves > 1


def test_batch_matches_oracle(batch):
    ctx, jobs, keep = batch
    st = ctx.render_batch(jobs[:2], abi.PT_BATCH_NO_TUNE | abi.PT_BATCH_CAPACITY_LOG2(11))
    for j in range(2):
        img, _ = oracle.OracleScene(keep[j][1]).render(jobs[j][1])
        assert _same(ctx.read_batch_image(j), img), j


def test_graph_and_tuning_are_reused(batch):
    ctx, jobs, _ = batch
    a = ctx.render_batch(jobs, abi.PT_BATCH_RETUNE)
    imgs = [ctx.read_batch_image(j).copy() for j in range(len(jobs))]
    b = ctx.render_batch(jobs, 0)
    assert a.graph_reused == 0 and a.tune_milliseconds > 0
    assert b.graph_reused == 1 and b.tune_milliseconds == 0 and b.build_milliseconds == 0
    assert (b.wave_capacity, b.tile_w, b.mega_threshold) == (a.wave_capacity, a.tile_w, a.mega_threshold)
    for j in range(len(jobs)):
        assert _same(ctx.read_batch_image(j), imgs[j])


def test_megakernel_jobs_beside_the_waves(batch):
    ctx, jobs, _ = batch
    ref = _single(jobs)
    mixed = []
    for i, (c, p) in enumerate(jobs):
        q = abi.RenderParams.from_buffer_copy(p)
        q.kernel = abi.PT_KERNEL_MEGA if i % 2 else abi.PT_KERNEL_WAVEFRONT
        mixed.append((c, q))
    for flags in (abi.PT_BATCH_NO_TUNE | abi.PT_BATCH_NO_GRAPH, abi.PT_BATCH_NO_TUNE):
        st = ctx.render_batch(mixed, flags)
        assert st.mega_jobs == len(jobs) // 2
        for j in range(len(jobs)):
            assert _same(ctx.read_batch_image(j), ref[j]), j


def test_fp64_sums(batch):
    ctx, jobs, _ = batch
    c, p = jobs[0]
    q = abi.RenderParams.from_buffer_copy(p)
    q.accum_mode = abi.PT_ACCUM_FP32_FP64
    c.render(q)
    single = c.read_image(fp64=True)
    ctx.render_batch([(c, q)] + jobs[1:3], abi.PT_BATCH_NO_TUNE)
    assert np.array_equal(ctx.read_batch_image(0, fp64=True), single)
    with pytest.raises(P.PtError):
        ctx.read_batch_image(1, fp64=True)


def test_same_scene_several_cameras(batch):
    """Jobs may share a scene; the batch context itself may hold one."""
    ctx, jobs, keep = batch
    hs, view = keep[2]
    ctx.upload(view)
    ctx.build_accel()
    ps = []
    for w, h, spp in ((48, 32, 3), (32, 48, 5), (40, 40, 2)):
        ps.append((ctx, hs.render_params(w, h, spp, 4)))
    ref = _single(ps)
    ctx.render_batch(ps, abi.PT_BATCH_NO_TUNE | abi.PT_BATCH_CAPACITY_LOG2(12))
    for j in range(3):
        assert _same(ctx.read_batch_image(j), ref[j])


def test_refractive_and_textured_jobs_in_a_batch(batch):
    """Jobs whose scenes use the refractive dielectric and every texture map
    kind, packed with the others into multi-wave batches on two wave states,
    equal their single renders and the oracle."""
    ctx, jobs, _ = batch
    extra, keep = [], []
    for raw, cam in (scenes.glass_raw("glass"), scenes.textured_raw()):
        hs = P.HostScene.from_raw(raw, cam)
        view = hs.pack()
        c = P.Context(0)
        c.upload(view)
        c.build_accel()
        keep.append((hs, view, c))
        extra.append((c, hs.render_params(48, 40, 4, 8)))
    mixed = extra + jobs[:3]
    ref = _single(mixed)
    for flags in (abi.PT_BATCH_NO_TUNE | abi.PT_BATCH_CAPACITY_LOG2(12), abi.PT_BATCH_NO_TUNE):
        st = ctx.render_batch(mixed, flags)
        assert st.error_word == 0
        for j in range(len(mixed)):
            assert _same(ctx.read_batch_image(j), ref[j]), (flags, j)
    for k, (_, view, _) in enumerate(keep):  # the first jobs of `mixed` are the extra ones
        want, _ = oracle.OracleScene(view).render(extra[k][1])
        assert _same(ref[k], want), k
    for _, _, c in keep:
        c.close()


def test_invalid_batches(batch):
    ctx, jobs, _ = batch
    c, p = jobs[0]
    bad = abi.RenderParams.from_buffer_copy(p)
    bad.sample_index = 1
    with pytest.raises(P.PtError) as e:
        ctx.render_batch([(c, bad)])
    assert e.value.status == abi.PT_ERR_INVALID
    big = abi.RenderParams.from_buffer_copy(p)
    big.width, big.height = 4096, 4096
    with pytest.raises(P.PtError) as e:
        ctx.render_batch([(c, big)], abi.PT_BATCH_NO_TUNE)
    assert e.value.status == abi.PT_ERR_UNSUPPORTED
    small = abi.RenderParams.from_buffer_copy(p)
    with pytest.raises(P.PtError) as e:  # 40x32 pixels do not fit 2^10 paths
        ctx.render_batch([(c, small)], abi.PT_BATCH_NO_TUNE | abi.PT_BATCH_CAPACITY_LOG2(10))
    assert e.value.status == abi.PT_ERR_UNSUPPORTED
    fresh = P.Context(0)
    with pytest.raises(P.PtError) as e:
        ctx.render_batch([(fresh, p)])
    assert e.value.status == abi.PT_ERR_STATE
    fresh.close()


def test_batch_job_times(batch):
    """pt_batch_job_times: each job's completion time of the last batch, within
    the batch's device time; waves take the least work first, so the smallest
    job is final no later than the largest."""
    ctx, jobs, _ = batch
    st = ctx.render_batch(jobs, abi.PT_BATCH_NO_TUNE | abi.PT_BATCH_CAPACITY_LOG2(13))
    assert st.waves > 1
    t = ctx.batch_job_times()
    assert t.shape == (len(jobs),) and (t > 0).all() and (t <= st.milliseconds * 1.01 + 0.05).all()
    work = [w * h * s for _, _, w, h, s, _ in SPECS]
    assert t[int(np.argmin(work))] <= t[int(np.argmax(work))]
    out = np.zeros(len(jobs) - 1, np.float32)
    rc = abi.lib().pt_batch_job_times(ctx._h, out.ctypes.data_as(C.POINTER(C.c_float)), len(jobs) - 1)
    assert rc == abi.PT_ERR_INVALID  # the count must be the last batch's
