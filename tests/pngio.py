"""Minimal 8-bit PNG / PGM / .flo helpers for the tests (stdlib zlib only)."""
from __future__ import annotations

import struct
import zlib

import numpy as np


def _chunk(tag, body):
    c = struct.pack(">I", len(body)) + tag + body
    return c + struct.pack(">I", zlib.crc32(tag + body) & 0xFFFFFFFF)


def write_png(path, img):
    img = np.ascontiguousarray(img, np.uint8)
    h, w = img.shape[:2]
    ctype = 0 if img.ndim == 2 else 2
    rows = b"".join(b"\x00" + img[y].tobytes() for y in range(h))
    data = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
    data += _chunk(b"IDAT", zlib.compress(rows, 6)) + _chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(data)


def read_png_rgb(path):
    with open(path, "rb") as f:
        data = f.read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h, ctype = 8, b"", 0, 0, 0
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    ch = {0: 1, 2: 3, 6: 4}[ctype]
    raw = zlib.decompress(idat)
    stride = w * ch
    out = np.zeros((h, stride), np.uint8)
    for y in range(h):
        assert raw[y * (stride + 1)] == 0  # the CLI writes filter 0
        out[y] = np.frombuffer(raw[y * (stride + 1) + 1:(y + 1) * (stride + 1)], np.uint8)
    return out.reshape(h, w, ch)


def write_pgm(path, img):
    img = np.ascontiguousarray(img, np.uint8)
    h, w = img.shape
    with open(path, "wb") as f:
        f.write(b"P5\n%d %d\n255\n" % (w, h) + img.tobytes())


def read_flo(path):
    with open(path, "rb") as f:
        tag = struct.unpack("<f", f.read(4))[0]
        assert tag == 202021.25
        w, h = struct.unpack("<ii", f.read(8))
        a = np.frombuffer(f.read(), np.float32).reshape(h, w, 2)
    return a[..., 0].copy(), a[..., 1].copy()


def write_flo(path, u, v):
    h, w = u.shape
    a = np.stack([u, v], axis=-1).astype(np.float32)
    with open(path, "wb") as f:
        f.write(struct.pack("<f", 202021.25) + struct.pack("<ii", w, h) + a.tobytes())
