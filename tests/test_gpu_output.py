"""Output stage on the GPU: tone map, device meansq and the `pt` CLI end to end,
checked against the oracle."""
import ctypes as C
import re
import struct
import subprocess
import zlib

import numpy as np
import pytest

import oracle
import pt_gb300 as P
from pt_gb300 import abi, scenes
from pt_gb300.build import CLI

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small(tmp_path_factory):
    d = tmp_path_factory.mktemp("small")
    path = scenes.small_scene(d, seed=0)
    hs = P.HostScene.load(path)
    return path, hs, hs.pack()


def png_pixels(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if typ == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    assert (raw[:, 0] == 0).all()
    return raw[:, 1:].reshape(h, w, 4)


def test_tonemap_matches_oracle(small):
    _, hs, view = small
    with P.Context(0) as ctx:
        ctx.upload(view)
        ctx.build_accel()
        ctx.render(hs.render_params(80, 60, 4, 6))
        lin = ctx.read_image().copy()
        ctx.tonemap()
        gpu = ctx.read_image()
    ref = lin.copy()
    oracle.lib().or_tonemap(oracle.fptr(ref), ref.shape[0] * ref.shape[1])
    # powf of the device and of the host C library differ by a few ulp
    assert np.max(np.abs(gpu - ref)) < 2e-6
    assert np.array_equal(gpu[..., 3], lin[..., 3])
    q_gpu = np.clip(gpu * 255.0, 0, 255).astype(np.uint8)
    q_ref = np.clip(ref * 255.0, 0, 255).astype(np.uint8)
    assert np.mean(q_gpu != q_ref) < 1e-3


def test_device_meansq_matches_oracle(small):
    _, hs, view = small
    with P.Context(0) as ctx:
        ctx.upload(view)
        ctx.build_accel()
        ctx.render(hs.render_params(96, 64, 16, 6))
        ref = ctx.read_image().copy()
        ctx.render(hs.render_params(96, 64, 2, 6))
        img = ctx.read_image().copy()
        mse = ctx.mse(ref)
    expect = oracle.meansq(ref, img)
    assert expect > 0
    assert abs(mse - expect) <= 1e-12 * expect


def test_cli_hdr_output_equals_oracle(small, tmp_path):
    path, hs, view = small
    out = tmp_path / "out.hdr"
    r = subprocess.run([str(CLI), "--headless", "-w", "64", "-h48", "-s", "4", "-b", "5", "-o", str(out), "-f", "hdr",
                        str(path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Scene has:" in r.stdout
    assert re.search(r"Rendering took [0-9.e+-]+ seconds with 4 samples taken per pixel\.", r.stdout)
    assert re.search(r"[0-9.e+-]+ samples per second\.", r.stdout)
    assert f"Writing image to {out}" in r.stdout
    ref, _ = oracle.OracleScene(view).render(hs.render_params(64, 48, 4, 5))
    expect = tmp_path / "oracle.hdr"
    assert abi.lib().pt_write_hdr(str(expect).encode(), oracle.fptr(ref), 64, 48) == 0
    assert out.read_bytes() == expect.read_bytes()


def test_cli_png_output_matches_oracle(small, tmp_path):
    path, hs, view = small
    out = tmp_path / "out.png"
    r = subprocess.run([str(CLI), "--headless", "-w", "64", "-h", "48", "-s", "4", "-b", "5", "-o", str(out), str(path)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    ref, _ = oracle.OracleScene(view).render(hs.render_params(64, 48, 4, 5))
    oracle.lib().or_tonemap(oracle.fptr(ref), 64 * 48)
    expect = np.clip(ref * 255.0, 0, 255).astype(np.uint8)
    got = png_pixels(out)
    diff = np.abs(got.astype(int) - expect.astype(int))
    assert diff.max() <= 1 and np.mean(diff != 0) < 1e-3
