"""The per-segment algorithmic byte counts used by bench.py's roofline come
from the oracle's binned-SAH BVH2 on the first sample of each scene."""
import sys
from pathlib import Path

import pytest

import oracle
import pt_gb300 as P
from pt_gb300 import scenes

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
import bench  # noqa: E402


@pytest.mark.parametrize("name,fn,w,h", [("small", scenes.small_scene, 256, 256), ("mid", scenes.mid_scene, 1024, 1024)])
def test_bseg_constants(tmp_path, name, fn, w, h):
    hs = P.HostScene.load(fn(tmp_path / name))
    view = hs.pack()
    _, st = oracle.OracleScene(view).render(hs.render_params(w, h, 1, 8))
    got = {"n_node": st.node_visits / st.ray_count, "n_tri": st.tri_tests / st.ray_count, "p_nee": st.shadow_rays / st.segments}
    for k, v in got.items():
        assert abs(v - bench.BSEG[name][k]) < 1e-3, (k, v)
    assert 1500 < bench.bseg_bytes(bench.BSEG[name]) < 5000


def test_bseg_constants_heavy():
    """The heavy configuration: 1920x1080, first sample, 12 bounces, Russian
    roulette from segment 4."""
    raw, cam = scenes.heavy_scene()
    hs = P.HostScene.from_raw(raw, cam)
    _, st = oracle.OracleScene(hs.pack()).render(hs.render_params(1920, 1080, 1, 12, rr_start=4))
    got = {"n_node": st.node_visits / st.ray_count, "n_tri": st.tri_tests / st.ray_count, "p_nee": st.shadow_rays / st.segments}
    for k, v in got.items():
        assert abs(v - bench.BSEG["heavy"][k]) < 1e-3, (k, v)
