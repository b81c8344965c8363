"""Parity of the CUDA path with the oracle at the benchmark configurations'
own sizes, not crops:

  small  256x256, 16 spp, 8 bounces, seed 0: the whole render, both kernels;
  mid    1024x1024, 8 bounces, thin lens: the first two samples of a
         128-spp render (sample indices 0-1) and its last two (126-127),
         the latter restarted at 126 so the running mean holds only them;
  heavy  1920x1080, 12 bounces, Russian roulette from segment 4: the full
         frame on the GPU at sample 0 and at sample 255 (the last of 256),
         compared on bands of rows that the oracle renders with the film
         coordinates of the real frame;
  batch  the 64-job batch workload (sides 128-1024, 4-256 spp, 1k-500k
         triangles) rendered as one tuned, graph-launched batch; three of its
         jobs rendered by the oracle in full.

Every compared value must be equal bit for bit (the tracer's stated
tolerance is 0 ulp), and where the oracle renders the whole image, the
traced segment and shadow-ray counts must be equal too.  The sample indices
enter the Sobol' sampler directly (pathtrace.rg.hlsl:13-16, the global
`sample_index`; sample.hlsli:94-166), so late indices exercise other sampler
states than the first samples do.
"""
import numpy as np
import pytest

import oracle
import pt_gb300 as P
from pt_gb300 import abi, replicas, scenes

pytestmark = pytest.mark.gpu

KERNELS = {"mega": abi.PT_KERNEL_MEGA, "wave": abi.PT_KERNEL_WAVEFRONT}


@pytest.fixture(scope="module")
def ctx():
    c = P.Context(0)
    yield c
    c.close()


def _assert_bitexact(gpu, ref, what=""):
    diff = gpu.view(np.uint32) != ref.view(np.uint32)
    if diff.any():
        ys, xs = np.nonzero(diff.reshape(gpu.shape[0], gpu.shape[1], -1).any(-1))
        raise AssertionError(f"{what}: {len(ys)} pixels differ (first at x={xs[0]}, y={ys[0]})")


@pytest.mark.parametrize("kernel", sorted(KERNELS))
def test_small_config_full_render(ctx, tmp_path, kernel):
    hs = P.HostScene.load(scenes.small_scene(tmp_path, seed=0))
    view = hs.pack()
    params = hs.render_params(256, 256, 16, 8, kernel=KERNELS[kernel])
    ctx.upload(view)
    ctx.build_accel()
    st = ctx.render(params)
    assert st.error_word == 0 and st.paths == 256 * 256 * 16
    gpu = ctx.read_image()
    ref, ost = oracle.OracleScene(view).render(params)
    _assert_bitexact(gpu, ref, "small 256x256x16")
    assert st.segments == ost.segments and st.shadow_rays == ost.shadow_rays


@pytest.fixture(scope="module")
def mid(tmp_path_factory):
    hs = P.HostScene.load(scenes.mid_scene(tmp_path_factory.mktemp("mid"), seed=1))
    view = hs.pack()
    return hs, view, oracle.OracleScene(view)


@pytest.mark.parametrize("first", [0, 126])
def test_mid_config_full_frame_first_and_last_samples(ctx, mid, first):
    hs, view, osc = mid
    params = hs.render_params(1024, 1024, 2, 8, sample_index=first, accum_mode=abi.PT_ACCUM_FP32_FP64)
    params.flags = abi.PT_RENDER_RESTART
    ctx.upload(view)
    ctx.build_accel()
    st = ctx.render(params)
    assert st.error_word == 0
    gpu = ctx.read_image()
    g64 = replicas.read_sums(ctx)
    s64 = np.zeros((1024, 1024, 4), np.float64)
    ref, ost = osc.render(params, sum64=s64)
    _assert_bitexact(gpu, ref, f"mid 1024x1024, samples {first}-{first + 1}")
    assert np.array_equal(g64[..., 3], s64[..., 3])
    # both sides add the same two FP32 values per pixel into FP64 sums in sample order
    assert np.array_equal(g64[..., :3], s64[..., :3])
    assert st.segments == ost.segments and st.shadow_rays == ost.shadow_rays


@pytest.fixture(scope="module")
def heavy():
    raw, cam = scenes.heavy_scene()
    hs = P.HostScene.from_raw(raw, cam)
    view = hs.pack()
    return hs, view, oracle.OracleScene(view)


# bands of rows at the top, middle and bottom of the 1080-row frame
HEAVY_BANDS = [(0, 24), (528, 552), (1056, 1080)]


@pytest.mark.parametrize("first", [0, 255])
def test_heavy_config_full_hd_row_bands(ctx, heavy, first):
    hs, view, osc = heavy
    params = hs.render_params(1920, 1080, 1, 12, sample_index=first, rr_start=4)
    params.flags = abi.PT_RENDER_RESTART
    ctx.upload(view)
    ctx.build_accel()
    st = ctx.render(params)
    assert st.error_word == 0 and st.paths == 1920 * 1080
    gpu = ctx.read_image()
    ref = np.zeros((1080, 1920, 4), np.float32)
    for r0, r1 in HEAVY_BANDS:
        osc.render(params, rgba=ref, rows=(r0, r1))
        _assert_bitexact(gpu[r0:r1], ref[r0:r1], f"heavy 1920x1080 sample {first}, rows {r0}-{r1}")


def test_batch_config_jobs_match_oracle():
    spec = scenes.batch_workload()
    ctx = P.Context(0)
    keep, jobs = [], []
    try:
        for j in spec:
            raw, cam = scenes.batch_scene(j["seed"], j["tris"])
            hs = P.HostScene.from_raw(raw, cam)
            view = hs.pack()
            c = P.Context(0)
            c.upload(view)
            c.build_accel()
            keep.append((hs, view))
            jobs.append((c, hs.render_params(j["side"], j["side"], j["spp"], j["max_bounces"])))
        st = ctx.render_batch(jobs)
        assert st.error_word == 0
        assert st.paths == sum(j["side"] ** 2 * j["spp"] for j in spec)
        # the three jobs with the fewest path samples, rendered whole by the oracle
        picks = sorted(range(len(spec)), key=lambda k: spec[k]["side"] ** 2 * spec[k]["spp"])[:3]
        for k in picks:
            img, _ = oracle.OracleScene(keep[k][1]).render(jobs[k][1])
            _assert_bitexact(ctx.read_batch_image(k), img, f"batch job {k} ({spec[k]})")
    finally:
        for c, _ in jobs:
            c.close()
        ctx.close()
