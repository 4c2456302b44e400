"""Film post-processing and image output on the CPU: the PNG writer
(pt_write_png, read back with zlib) and the oracle's restatement of
FrameBuffer::gaussianBlur (framebuffer.cpp:60-129)."""
from __future__ import annotations

import struct
import zlib

import numpy as np

from oracle import pyoracle as O
from pathtracer_gb300 import native as N


def _read_png(path):
    data = path.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat = 8, b""
    w = h = None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        assert crc == zlib.crc32(typ + body) & 0xffffffff
        if typ == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert (depth, ctype) == (8, 2)
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 3 * w)
    assert np.all(rows[:, 0] == 0)
    return rows[:, 1:].reshape(h, w, 3)


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    for w, h in ((1, 1), (37, 23), (300, 250)):  # the last spans several stored blocks
        img = rng.integers(0, 256, size=(h, w, 3), dtype=np.uint8)
        p = tmp_path / f"img_{w}x{h}.png"
        N.write_png(p, img)
        assert np.array_equal(_read_png(p), img)


def test_oracle_blur_properties():
    rng = np.random.default_rng(2)
    const = np.full((9, 11, 3), 0.25, np.float32)
    out = O.gaussian_blur(const, 5, 1.5)
    assert np.allclose(out, 0.25, rtol=1e-6)
    film = rng.random((9, 11, 3), dtype=np.float32)
    for k, s in ((4, 1.0), (1, 1.0), (5, -1.0)):  # refused as the reference refuses them
        assert np.array_equal(O.gaussian_blur(film, k, s), film)
    blurred = O.gaussian_blur(film, 3, 0.8)
    assert blurred.std() < film.std()
