"""pt_mse_noalloc: the meansq reduction for callers that cannot allocate device
memory (host applications that own all device memory and forbid allocations in
plug-ins, processes under a hard device-memory cap, real-time loops that must
avoid cudaMalloc's implicit synchronisation).

It must give the value of the existing entry point pt_mse_host for the same
images, call after call, while its scratch lives in a fixed array inside the
library.  The images are caller-owned device buffers (torch allocates them
here, on the caller's side).  This file is collected last so that a run that
stops at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import pt_gb300 as P
from pt_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def _noalloc(img_dev, ref_dev, w, h, out_dev):
    return abi.lib().pt_mse_noalloc(C.c_void_p(img_dev.data_ptr()), C.c_void_p(ref_dev.data_ptr()), w, h,
                                    C.c_void_p(out_dev.data_ptr()), None)


def test_noalloc_matches_existing_entry_point_twice(tmp_path):
    torch = pytest.importorskip("torch")
    hs = P.HostScene.load(scenes.small_scene(tmp_path, seed=0))
    view = hs.pack()
    w, h = 96, 80
    with P.Context(0) as ctx:
        ctx.upload(view)
        ctx.build_accel()
        ctx.render(hs.render_params(w, h, 16, 6))
        reference = ctx.read_image().copy()
        images = []
        for spp in (1, 3):
            ctx.render(hs.render_params(w, h, spp, 6))
            images.append((ctx.read_image().copy(), ctx.mse(reference)))
    ref_dev = torch.from_numpy(reference).cuda()
    out = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for img, expected in images:
        img_dev = torch.from_numpy(img).cuda()
        torch.cuda.synchronize()
        # two calls in a row on the same inputs, each into its own output
        assert _noalloc(img_dev, ref_dev, w, h, out[0:1]) == abi.PT_OK
        assert _noalloc(img_dev, ref_dev, w, h, out[1:2]) == abi.PT_OK
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert expected > 0
        # the same reduction as pt_mse_host: same grid, same order of sums
        assert got[0] == expected and got[1] == expected


def test_noalloc_rejects_bad_arguments():
    torch = pytest.importorskip("torch")
    a = torch.zeros((4, 4, 4), dtype=torch.float32, device="cuda")
    out = torch.zeros((1,), dtype=torch.float64, device="cuda")
    L = abi.lib()
    assert L.pt_mse_noalloc(None, C.c_void_p(a.data_ptr()), 4, 4, C.c_void_p(out.data_ptr()), None) == abi.PT_ERR_INVALID
    assert L.pt_mse_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(a.data_ptr()), 0, 4, C.c_void_p(out.data_ptr()), None) \
        == abi.PT_ERR_INVALID
    assert L.pt_mse_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(a.data_ptr()), 65536, 65536, C.c_void_p(out.data_ptr()),
                            None) == abi.PT_ERR_UNSUPPORTED
    assert L.pt_mse_noalloc(C.c_void_p(a.data_ptr() + 4), C.c_void_p(a.data_ptr()), 2, 2, C.c_void_p(out.data_ptr()),
                            None) == abi.PT_ERR_INVALID
    # an output that is not 8-byte aligned (a byte offset into a device buffer)
    assert L.pt_mse_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(a.data_ptr()), 2, 2, C.c_void_p(out.data_ptr() + 4),
                            None) == abi.PT_ERR_INVALID
    torch.cuda.synchronize()
