"""Checkpoint / resume logic on CPU: chunked progressive renders written to
disk and resumed, the fingerprint guard, and training-state files.  The
context here is a stand-in whose renders are the oracle's (the GPU renders
the same samples bit for bit, tests/test_gpu_parity.py); the GPU path
itself is covered by tests/test_gpu_checkpoint.py."""
import numpy as np
import pytest

import oracle
import pt_gb300 as P
from pt_gb300 import abi, checkpoint, replicas, scenes

W, H = 20, 12


class OracleCtx:
    """Holds a running mean and FP64 sums like a context; renders with the oracle."""

    def __init__(self, view):
        self.orc = oracle.OracleScene(view, brute_force=True)
        self.rgba = np.zeros((H, W, 4), np.float32)
        self.s64 = np.zeros((H, W, 4), np.float64)
        self.renders = 0

    def render(self, p, stats=True):
        assert p.accum_mode == abi.PT_ACCUM_FP32_FP64
        if p.sample_index == 0:
            self.rgba[:] = 0
            self.s64[:] = 0
        self.orc.render(p, rgba=self.rgba, sum64=self.s64)
        self.renders += 1

    def read_image(self):
        return self.rgba.copy()

    def restore_image(self, rgba, samples_done, sums64=None):
        self.rgba[:] = rgba
        self.s64[:] = sums64


@pytest.fixture()
def scene(monkeypatch):
    monkeypatch.setattr(replicas, "read_sums", lambda ctx: ctx.s64.copy())
    raw, cam = scenes.tiny_raw("two_tris")
    hs = P.HostScene.from_raw(raw, cam)
    return hs, hs.pack()


def test_progressive_render_resumes_exactly(scene, tmp_path):
    hs, view = scene
    p = hs.render_params(W, H, 1, 3)
    whole = OracleCtx(view)
    assert checkpoint.render_progressive(whole, view, p, 7, tmp_path / "whole.npz", chunk=7) == 7
    path = tmp_path / "ck.npz"
    a = OracleCtx(view)
    assert checkpoint.render_progressive(a, view, p, 7, path, chunk=2, stop_after=2) == 4
    assert not (tmp_path / "ck.npz.tmp").exists()
    b = OracleCtx(view)  # a new process picks the file up
    assert checkpoint.render_progressive(b, view, p, 7, path, chunk=2) == 7
    assert b.renders == 2  # samples 4-5 and 6
    assert np.array_equal(b.rgba.view(np.uint32), whole.rgba.view(np.uint32))
    assert np.array_equal(b.s64, whole.s64)
    # a finished checkpoint renders nothing more
    c = OracleCtx(view)
    assert checkpoint.render_progressive(c, view, p, 7, path, chunk=2) == 7 and c.renders == 0
    with pytest.raises(ValueError, match="more than"):
        checkpoint.render_progressive(OracleCtx(view), view, p, 5, path)


def test_fingerprint_guards_scene_and_settings(scene, tmp_path):
    hs, view = scene
    p = hs.render_params(W, H, 1, 3)
    path = tmp_path / "ck.npz"
    checkpoint.render_progressive(OracleCtx(view), view, p, 2, path, chunk=2)
    f0 = checkpoint.render_fingerprint(view, p)
    q = abi.RenderParams.from_buffer_copy(p)
    q.sample_index, q.samples, q.kernel = 5, 9, abi.PT_KERNEL_MEGA
    assert checkpoint.render_fingerprint(view, q) == f0  # sample range and kernel do not matter
    q.max_bounces = 4
    assert checkpoint.render_fingerprint(view, q) != f0
    with pytest.raises(ValueError, match="another scene"):
        checkpoint.render_progressive(OracleCtx(view), view, q, 4, path)
    raw, cam = scenes.tiny_raw("two_tris")
    raw = {k: (v.copy() if hasattr(v, "copy") else v) for k, v in raw.items()}
    raw["vertices"][0, 0] += 0.25
    hs2 = P.HostScene.from_raw(raw, cam)
    assert checkpoint.render_fingerprint(hs2.pack(), p) != f0


class FakeNet:
    def __init__(self, n):
        self.p = np.zeros(n, np.float32)
        self.m = np.zeros(n, np.float32)
        self.v = np.zeros(n, np.float32)
        self.t = 0

    def params(self):
        return self.p.copy()

    def set_params(self, p):
        self.p[:] = p
        self.m[:] = 0
        self.v[:] = 0
        self.t = 0

    def adam_state(self):
        return self.m.copy(), self.v.copy(), self.t

    def set_adam_state(self, m, v, t):
        self.m[:], self.v[:], self.t = m, v, t


def test_training_state_round_trip(tmp_path):
    import torch

    rng = np.random.default_rng(3)
    a = FakeNet(1000)
    a.p[:] = rng.standard_normal(1000)
    a.m[:] = rng.standard_normal(1000)
    a.v[:] = rng.random(1000)
    a.t = 1234
    gen = torch.Generator().manual_seed(7)
    torch.randint(0, 100, (16,), generator=gen)
    path = tmp_path / "train.npz"
    checkpoint.save_training(path, a, 1234, gen.get_state(), {"seed": 7})
    want = torch.randint(0, 100, (16,), generator=gen)
    b = FakeNet(1000)
    step, rng_state, meta = checkpoint.load_training(path, b)
    assert step == 1234 and meta == {"seed": 7}
    assert np.array_equal(b.p, a.p) and np.array_equal(b.m, a.m) and np.array_equal(b.v, a.v) and b.t == 1234
    g2 = torch.Generator()
    g2.set_state(torch.from_numpy(rng_state))
    assert torch.equal(torch.randint(0, 100, (16,), generator=g2), want)
