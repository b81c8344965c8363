"""A small baseline JPEG writer (ITU-T T.81 sequential Huffman mode) for test
fixtures: greyscale or three-component YCbCr images with chosen sampling
factors and restart intervals, forms the reference's own JPEG writer
(stb_image_write: 4:4:4 or 4:2:0, no restarts, always three components) does
not produce.  Used only by make_golden.py; the fixtures it makes are decoded
by the reference's stb_image to give the expected texels.

Entropy tables are simple valid canonical codes (every DC size category 4
bits long, every AC run/size symbol 8 bits long), the quantisation table a
ramp over the zig-zag order; the forward DCT is the exact 2-D DCT of T.81
A.3.3 in double precision.
"""
from __future__ import annotations

import math

import numpy as np


def _zigzag() -> list[int]:
    out = []
    for s in range(15):
        lo, hi = max(0, s - 7), min(7, s)
        rows = range(lo, hi + 1) if s & 1 else range(hi, lo - 1, -1)
        out += [r * 8 + (s - r) for r in rows]
    return out


ZIGZAG = _zigzag()
_C = np.array([[(math.sqrt(0.5) if u == 0 else 1.0) * 0.5 * math.cos((2 * x + 1) * u * math.pi / 16)
                for x in range(8)] for u in range(8)])

DC_SYMBOLS = list(range(12))
AC_SYMBOLS = [0x00, 0xF0] + [(r << 4) | s for r in range(16) for s in range(1, 11)]


class _Bits:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, value: int, length: int):
        for i in range(length - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc, self.n = 0, 0

    def flush(self):
        while self.n:
            self.put(1, 1)  # pad with 1-bits


def _codes(symbols, length):
    return {s: (i, length) for i, s in enumerate(symbols)}


def _dht(tc, th, symbols, length):
    counts = [0] * 16
    counts[length - 1] = len(symbols)
    body = bytes([(tc << 4) | th]) + bytes(counts) + bytes(symbols)
    return b"\xFF\xC4" + (len(body) + 2).to_bytes(2, "big") + body


def _category(v: int) -> int:
    return 0 if v == 0 else int(abs(v)).bit_length()


def _encode_block(bits, block, q, pred, dc, ac):
    """block: 8x8 level-shifted samples; returns the new DC prediction."""
    coef = _C @ block @ _C.T  # F[v][u] = sum_y sum_x c[v][y] c[u][x] s[y][x]
    zz = [int(round(coef.flat[ZIGZAG[k]] / q[k])) for k in range(64)]
    diff = zz[0] - pred
    s = _category(diff)
    bits.put(*dc[s])
    if s:
        bits.put(diff if diff > 0 else diff + (1 << s) - 1, s)
    run = 0
    for k in range(1, 64):
        v = zz[k]
        if v == 0:
            run += 1
            continue
        while run > 15:
            bits.put(*ac[0xF0])
            run -= 16
        s = _category(v)
        bits.put(*ac[(run << 4) | s])
        bits.put(v if v > 0 else v + (1 << s) - 1, s)
        run = 0
    if run:
        bits.put(*ac[0x00])
    return zz[0]


def encode(img: np.ndarray, sampling=(1, 1), restart: int = 0, rgb_ids: bool = False) -> bytes:
    """img: uint8 [h, w] (greyscale) or [h, w, 3] (RGB, stored as YCbCr, or as
    RGB with component ids 'R','G','B' when rgb_ids).  sampling = (H, V) of
    the luma component (chroma is 1x1)."""
    img = np.asarray(img, np.float64)
    h, w = img.shape[:2]
    q = [2 + k // 4 for k in range(64)]
    if img.ndim == 2:
        planes, factors = [img], [(1, 1)]
        ids = [1]
    else:
        r, g, b = img[..., 0], img[..., 1], img[..., 2]
        if rgb_ids:
            planes, ids = [r, g, b], [ord("R"), ord("G"), ord("B")]
        else:
            y = 0.299 * r + 0.587 * g + 0.114 * b
            cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128
            cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128
            planes, ids = [y, cb, cr], [1, 2, 3]
        factors = [sampling, (1, 1), (1, 1)]
    hmax = max(f[0] for f in factors)
    vmax = max(f[1] for f in factors)
    mcux, mcuy = -(-w // (8 * hmax)), -(-h // (8 * vmax))
    padded = []
    for p, (fh, fv) in zip(planes, factors):
        # pad the full-resolution plane to whole MCUs by edge replication, then subsample by averaging
        P = np.pad(p, ((0, mcuy * 8 * vmax - h), (0, mcux * 8 * hmax - w)), mode="edge")
        sh, sv = hmax // fh, vmax // fv
        P = P.reshape(P.shape[0] // sv, sv, P.shape[1] // sh, sh).mean(axis=(1, 3))
        padded.append(P - 128.0)
    out = bytearray(b"\xFF\xD8")
    out += b"\xFF\xDB" + (67).to_bytes(2, "big") + bytes([0]) + bytes(q)
    nf = len(planes)
    sof = bytes([8]) + h.to_bytes(2, "big") + w.to_bytes(2, "big") + bytes([nf])
    for i, (fh, fv) in zip(ids, factors):
        sof += bytes([i, (fh << 4) | fv, 0])
    out += b"\xFF\xC0" + (len(sof) + 2).to_bytes(2, "big") + sof
    out += _dht(0, 0, DC_SYMBOLS, 4) + _dht(1, 0, AC_SYMBOLS, 8)
    if restart:
        out += b"\xFF\xDD\x00\x04" + restart.to_bytes(2, "big")
    sos = bytes([nf]) + b"".join(bytes([i, 0x00]) for i in ids) + bytes([0, 63, 0])
    out += b"\xFF\xDA" + (len(sos) + 2).to_bytes(2, "big") + sos
    dc, ac = _codes(DC_SYMBOLS, 4), _codes(AC_SYMBOLS, 8)
    bits = _Bits()
    preds = [0] * nf
    total, count, rst = mcux * mcuy, 0, 0
    for my in range(mcuy):
        for mx in range(mcux):
            for c, (P, (fh, fv)) in enumerate(zip(padded, factors)):
                for v in range(fv):
                    for hh in range(fh):
                        by, bx = (my * fv + v) * 8, (mx * fh + hh) * 8
                        preds[c] = _encode_block(bits, P[by:by + 8, bx:bx + 8], q, preds[c], dc, ac)
            count += 1
            if restart and count % restart == 0 and count < total:
                bits.flush()
                out += bits.out
                bits.out = bytearray()
                out += bytes([0xFF, 0xD0 + rst])
                rst = (rst + 1) & 7
                preds = [0] * nf
    bits.flush()
    out += bits.out + b"\xFF\xD9"
    return bytes(out)
