"""The oracle's BVH traversal gives the exact closest hit: identical to testing
every triangle of every instance (brute force), for images and single rays."""
import numpy as np
import pytest

import oracle
import pt_gb300 as P
from pt_gb300 import scenes


@pytest.fixture(scope="module")
def small(tmp_path_factory):
    hs = P.HostScene.load(scenes.small_scene(tmp_path_factory.mktemp("s"), seed=0))
    return hs, hs.pack()


def test_bvh_equals_brute_force_image(small):
    hs, view = small
    params = hs.render_params(24, 24, 2, 6)
    a, sa = oracle.OracleScene(view).render(params)
    b, sb = oracle.OracleScene(view, brute_force=True).render(params)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert sa.segments == sb.segments and sa.shadow_rays == sb.shadow_rays
    assert sa.tri_tests < sb.tri_tests


def test_bvh_equals_brute_force_rays(small):
    hs, view = small
    bvh = oracle.OracleScene(view)
    brute = oracle.OracleScene(view, brute_force=True)
    rng = np.random.default_rng(1)
    hits = 0
    for _ in range(3000):
        o = rng.uniform(-6, 6, 3).astype(np.float32)
        o[1] = rng.uniform(0.05, 7)
        d = rng.normal(0, 1, 3).astype(np.float32)
        d /= np.linalg.norm(d)
        a = bvh.intersect(o.tolist(), d.tolist())
        b = brute.intersect(o.tolist(), d.tolist())
        assert a == b
        hits += a is not None
    assert hits > 1000


def test_axis_aligned_and_grazing_rays(small):
    """Rays with zero direction components and rays in the ground plane."""
    hs, view = small
    bvh = oracle.OracleScene(view)
    brute = oracle.OracleScene(view, brute_force=True)
    for o, d in [((0, 3, 0), (0, -1, 0)), ((0.5, 0.0, -9), (0, 0, 1)), ((-10, 0, -10), (1, 0, 0)),
                 ((10, 0, 10), (-1, 0, -1)), ((0, 6, 0), (0, 1, 0)), ((0, 6, 0), (0, -1, 0)), ((1, 1, 1), (0, 0, -1))]:
        assert bvh.intersect(o, d) == brute.intersect(o, d), (o, d)


def test_sincos_accuracy():
    L = oracle.lib()
    xs = np.concatenate([np.linspace(-7, 7, 20001), np.linspace(0, 2 * np.pi, 5003)]).astype(np.float32)
    s = np.array([L.or_sin(float(x)) for x in xs], np.float32)
    c = np.array([L.or_cos(float(x)) for x in xs], np.float32)
    ts = np.sin(xs.astype(np.float64))
    tc = np.cos(xs.astype(np.float64))
    ulp = np.spacing(np.float32(1.0))
    assert np.max(np.abs(s - ts)) < 4 * ulp
    assert np.max(np.abs(c - tc)) < 4 * ulp
    assert np.isnan(L.or_sin(float("nan"))) and np.isnan(L.or_cos(float("inf")))
