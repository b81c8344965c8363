"""Checkpoint / resume on the GPU: a progressive render cut into chunks,
saved to disk and resumed in new contexts equals the uninterrupted render
bit for bit; denoiser training resumed from a checkpoint (parameters, Adam
moments and step) continues where it stopped."""
import numpy as np
import pytest

import pt_gb300 as P
from pt_gb300 import abi, checkpoint, scenes
from pt_gb300.denoise import UNet, init_params

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_progressive_render_on_disk_resumes_bit_exactly(tmp_path):
    hs = P.HostScene.load(scenes.mid_scene(tmp_path / "m", seed=1))
    view = hs.pack()
    p = hs.render_params(96, 64, 1, 8)
    ref = P.Context(0)
    ref.upload(view)
    ref.build_accel()
    q = hs.render_params(96, 64, 37, 8, accum_mode=abi.PT_ACCUM_FP32_FP64)
    ref.render(q, stats=False)
    want = ref.read_image().copy()
    want64 = ref.read_image(fp64=True).copy()
    ref.close()
    path = tmp_path / "ck.npz"
    done = 0
    for _ in range(3):  # three "processes", two chunks of 8 samples each at most
        c = P.Context(0)
        c.upload(view)
        c.build_accel()
        done = checkpoint.render_progressive(c, view, p, 37, path, chunk=8, stop_after=2)
        got = c.read_image().copy()
        got64 = c.read_image(fp64=True).copy()
        c.close()
    assert done == 37
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(got64, want64)


def _batch(n, h, w, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0, 1, (n, h, w, 16)).astype(np.float32)
    x[..., 11:] = 0
    mix = rng.uniform(-0.5, 0.5, (16, 3))
    t = np.expm1(np.clip(x @ mix + 0.5, 0, 3)).astype(np.float32)
    t = np.concatenate([t, np.ones((n, h, w, 1), np.float32)], axis=-1)
    return (torch.from_numpy(x).to(torch.bfloat16).cuda(), torch.from_numpy(t).cuda())


def test_training_resume(tmp_path):
    n, h, w = 2, 32, 32
    data = [_batch(n, h, w, s) for s in range(6)]

    def step(net, i):
        x, t = data[i]
        net.input_tensor().copy_(x)
        net.forward()
        net.backward(t.data_ptr())
        net.adam(1e-3)

    p0 = init_params(2)
    a = UNet(n, h, w)
    a.set_params(p0)
    for i in range(3):
        step(a, i)
    path = tmp_path / "train.npz"
    gen = torch.Generator().manual_seed(0)
    checkpoint.save_training(path, a, 3, gen.get_state())
    m3, v3, t3 = a.adam_state()
    assert t3 == 3 and np.abs(m3).max() > 0 and v3.min() >= 0
    for i in range(3, 6):
        step(a, i)
    cont = a.params()

    b = UNet(n, h, w)
    b.set_params(init_params(9))
    s, _, _ = checkpoint.load_training(path, b)
    assert s == 3
    mb, vb, tb = b.adam_state()  # the state round-trips exactly
    assert tb == 3 and np.array_equal(mb, m3) and np.array_equal(vb, v3)
    for i in range(3, 6):
        step(b, i)
    resumed = b.params()

    # the same three steps from the saved parameters with the optimizer state lost
    c = UNet(n, h, w)
    c.set_params(np.load(path)["params"])
    for i in range(3, 6):
        step(c, i)
    lost = c.params()
    # weight gradients are summed with float atomics, so runs differ in the last bits
    drift = np.linalg.norm(resumed - cont)
    assert drift < 0.02 * np.linalg.norm(cont - p0), drift
    assert drift < 0.1 * np.linalg.norm(lost - cont), (drift, np.linalg.norm(lost - cont))
    for u in (a, b, c):
        u.close()
