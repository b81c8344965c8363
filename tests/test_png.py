"""PNG decoding for textures (CPU): every colour type and bit depth the
decoder accepts, all five scanline filters, stored / fixed / dynamic deflate
blocks and Adam7 interlace, against images encoded here with zlib.  Channel
counts follow what the reference asks stb_image for: the file's count with 3
widened to 4 (texturedata.cpp:30-48)."""
import ctypes as C
import struct
import zlib

import numpy as np
import pytest

from pt_gb300 import abi


def chunk(tag, data):
    c = struct.pack(">I", len(data)) + tag + data
    return c + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def filter_rows(raw, stride, bpp, ftypes):
    out, prev = bytearray(), bytearray(stride)
    for y in range(len(raw) // stride):
        row = raw[y * stride:(y + 1) * stride]
        ft = ftypes[y % len(ftypes)]
        f = bytearray(stride)
        for i in range(stride):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = [0, a, b, (a + b) >> 1, paeth(a, b, c)][ft]
            f[i] = (row[i] - pred) & 0xFF
        out += bytes([ft]) + f
        prev = row
    return bytes(out)


def pack_bits(vals, depth):
    out, acc, n = bytearray(), 0, 0
    for v in vals:
        acc = (acc << depth) | int(v)
        n += depth
        if n == 8:
            out.append(acc)
            acc, n = 0, 0
    if n:
        out.append(acc << (8 - n))
    return bytes(out)


def encode(img, ctype, depth=8, level=6, ftypes=(0, 1, 2, 3, 4), palette=None, trns=None, interlace=False):
    h, w = img.shape[:2]
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bpp = max(1, ch * depth // 8)

    def rows(sub):
        hh, ww = sub.shape[:2]
        raw = bytearray()
        for y in range(hh):
            r = sub[y].reshape(ww * ch)
            if depth < 8:
                raw += pack_bits(r, depth)
            elif depth == 16:
                raw += r.astype(">u2").tobytes()
            else:
                raw += r.astype(np.uint8).tobytes()
        stride = len(raw) // hh
        return filter_rows(bytes(raw), stride, bpp, ftypes)

    if interlace:
        data = b""
        for (ax, ay, sx, sy) in [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]:
            sub = img[ay::sy, ax::sx]
            if sub.shape[0] and sub.shape[1]:
                data += rows(sub)
    else:
        data = rows(img)
    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    if palette is not None:
        png += chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    if trns is not None:
        png += chunk(b"tRNS", bytes(trns))
    png += chunk(b"IDAT", zlib.compress(data, level)) + chunk(b"IEND", b"")
    return png


def decode(png):
    L = abi.lib()
    out = C.POINTER(C.c_uint8)()
    w, h, c, fc = C.c_uint32(), C.c_uint32(), C.c_uint32(), C.c_uint32()
    buf = C.create_string_buffer(png, len(png))
    rc = L.pt_png_decode(buf, len(png), C.byref(out), C.byref(w), C.byref(h), C.byref(c), C.byref(fc))
    if rc != abi.PT_OK:
        return rc, None, None
    arr = np.ctypeslib.as_array(out, shape=(h.value * w.value * c.value,)).copy().reshape(h.value, w.value, c.value)
    L.pt_host_free(out)
    return rc, arr, fc.value


RNG = np.random.default_rng(0)


@pytest.mark.parametrize("level", [0, 1, 9])
@pytest.mark.parametrize("interlace", [False, True])
def test_rgb_and_rgba(level, interlace):
    rgba = RNG.integers(0, 256, (13, 17, 4), dtype=np.uint8)
    rc, got, fc = decode(encode(rgba, 6, level=level, interlace=interlace))
    assert rc == 0 and fc == 4 and np.array_equal(got, rgba)
    rgb = rgba[..., :3]
    rc, got, fc = decode(encode(rgb, 2, level=level, interlace=interlace))
    assert rc == 0 and fc == 3 and got.shape[2] == 4
    assert np.array_equal(got[..., :3], rgb) and np.all(got[..., 3] == 255)


def test_gray_depths_and_alpha():
    for depth in (1, 2, 4, 8):
        g = RNG.integers(0, 1 << depth, (9, 11), dtype=np.uint16)
        rc, got, fc = decode(encode(g[..., None], 0, depth=depth))
        assert rc == 0 and fc == 1
        assert np.array_equal(got[..., 0], (g * 255 // ((1 << depth) - 1)).astype(np.uint8))
    ga = RNG.integers(0, 256, (7, 5, 2), dtype=np.uint8)
    rc, got, fc = decode(encode(ga, 4))
    assert rc == 0 and fc == 2 and np.array_equal(got, ga)


def test_sixteen_bit_keeps_high_byte():
    v = RNG.integers(0, 65536, (6, 8, 4), dtype=np.uint16)
    rc, got, _ = decode(encode(v, 6, depth=16))
    assert rc == 0 and np.array_equal(got, (v >> 8).astype(np.uint8))


def test_palette_with_transparency():
    pal = RNG.integers(0, 256, (16, 3), dtype=np.uint8)
    idx = RNG.integers(0, 16, (10, 12), dtype=np.uint8)
    for depth in (4, 8):
        rc, got, fc = decode(encode(idx[..., None], 3, depth=depth, palette=pal))
        assert rc == 0 and fc == 3 and np.array_equal(got[..., :3], pal[idx]) and np.all(got[..., 3] == 255)
    trns = list(range(0, 160, 10))
    rc, got, fc = decode(encode(idx[..., None], 3, palette=pal, trns=trns))
    assert rc == 0 and fc == 4 and np.array_equal(got[..., 3], np.array(trns, np.uint8)[idx])


def test_corrupt_input_is_an_error():
    good = encode(RNG.integers(0, 256, (4, 4, 4), dtype=np.uint8), 6)
    assert decode(b"not a png")[0] != 0
    assert decode(good[:40])[0] != 0
    bad = bytearray(good)
    bad[-20] ^= 0xFF  # inside the zlib stream
    assert decode(bytes(bad))[0] != 0 or True  # may still inflate; must not crash
