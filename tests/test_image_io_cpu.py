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


# ---------------------------------------------------------------- Radiance HDR
def _rle_channel(b: bytes) -> bytes:
    """Adaptive run-length encoding of one scanline channel (runs of 3+)."""
    out, i, n = bytearray(), 0, len(b)
    while i < n:
        j = i
        while j < n and j - i < 127 and b[j] == b[i]:
            j += 1
        if j - i >= 3:
            out += bytes([128 + j - i, b[i]])
            i = j
            continue
        k = i
        while k < n and k - i < 128 and not (k + 2 < n and b[k] == b[k + 1] == b[k + 2]):
            k += 1
        out += bytes([k - i]) + b[i:k]
        i = k
    return bytes(out)


def _write_hdr(path, rgbe: np.ndarray, rle: bool, magic=b"#?RADIANCE"):
    h, w, _ = rgbe.shape
    data = bytearray(magic + b"\n# made by the test\nFORMAT=32-bit_rle_rgbe\nEXPOSURE=1.0\n\n")
    data += f"-Y {h} +X {w}\n".encode()
    for y in range(h):
        if rle:
            data += bytes([2, 2, w >> 8, w & 255])
            for c in range(4):
                data += _rle_channel(rgbe[y, :, c].tobytes())
        else:
            data += rgbe[y].tobytes()
    path.write_bytes(bytes(data))


def _rgbe_to_float(rgbe: np.ndarray) -> np.ndarray:
    e = rgbe[..., 3].astype(np.int32)
    s = np.where(e > 0, np.ldexp(np.float32(1), e - 136), 0).astype(np.float32)
    return rgbe[..., :3].astype(np.float32) * s[..., None]


def _random_rgbe(rng, h, w):
    rgbe = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    rgbe[..., 3] = rng.integers(100, 160, (h, w))
    rgbe[h // 2, : w // 2] = rgbe[h // 2, 0]  # long runs for the RLE encoder
    rgbe[0, 0, 3] = 0                          # exponent 0: black
    return rgbe


def test_hdr_load_flat_and_rle(tmp_path):
    rng = np.random.default_rng(5)
    for (h, w), rle, magic in (((3, 5), False, b"#?RGBE"), ((16, 40), True, b"#?RADIANCE"),
                               ((9, 300), True, b"#?RADIANCE"), ((4, 7), True, b"#?RADIANCE")):
        rgbe = _random_rgbe(rng, h, w)
        p = tmp_path / f"img_{h}x{w}.hdr"
        _write_hdr(p, rgbe, rle and w >= 8, magic)
        want = _rgbe_to_float(rgbe)            # file rows, top first
        top_first = N.load_image(p, flip_y=True, hdr=True)
        bottom_first = N.load_image(p, flip_y=False, hdr=True)
        assert top_first.shape == (h, w, 3) and top_first.dtype == np.float32
        assert np.array_equal(top_first, want)
        assert np.array_equal(bottom_first, want[::-1])


def test_hdr_load_errors(tmp_path):
    import pytest
    with pytest.raises(N.PtError):
        N.load_image(tmp_path / "missing.hdr", hdr=True)
    bad = tmp_path / "bad.hdr"
    bad.write_bytes(b"P6\n1 1\n255\n\0\0\0")
    with pytest.raises(N.PtError):
        N.load_image(bad, hdr=True)
    rgbe = _random_rgbe(np.random.default_rng(0), 8, 16)
    _write_hdr(bad, rgbe, True)
    bad.write_bytes(bad.read_bytes()[:-9])  # truncated last run
    with pytest.raises(N.PtError):
        N.load_image(bad, hdr=True)


def test_hdr_texels_match_reference_image_texture(tmp_path):
    """Texel layout against the reference's own ImageTexture(isHDR = true)
    (stbi_loadf) through the reference harness, where it is built: at the
    lattice points u = x / W, v = y / H its bilinear getTexelColor returns
    texel (x, y) itself."""
    import pytest
    from oracle.ref import refbind
    if not refbind.available():
        pytest.skip("reference harness not built")
    rng = np.random.default_rng(9)
    h, w = 8, 16
    rgbe = _random_rgbe(rng, h, w)
    p = tmp_path / "env.hdr"
    _write_hdr(p, rgbe, True)
    xs, ys = np.meshgrid(np.arange(w - 1), np.arange(h - 1))
    uv = np.stack([xs.ravel() / w, ys.ravel() / h], 1).astype(np.float32)
    for flip in (False, True):
        ours = N.load_image(p, flip_y=flip, hdr=True)
        ref = refbind.image_texels(p, flip, True, uv)
        assert np.array_equal(ours[ys.ravel(), xs.ravel()], ref)


# ---------------------------------------------------------------- PNG reading
_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
_ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))


def _pack_row(samples: np.ndarray, depth: int) -> bytes:
    if depth == 16:
        return samples.astype(">u2").tobytes()
    if depth == 8:
        return samples.astype(np.uint8).tobytes()
    bits = np.unpackbits(samples.astype(np.uint8)[:, None], axis=1)[:, 8 - depth:].ravel()
    return np.packbits(bits).tobytes()


def _filter_row(raw: bytes, prev: bytes, bpp: int, f: int) -> bytes:
    out = bytearray([f])
    for i, x in enumerate(raw):
        a = raw[i - bpp] if i >= bpp else 0
        b = prev[i]
        c = prev[i - bpp] if i >= bpp else 0
        if f == 0:
            pred = 0
        elif f == 1:
            pred = a
        elif f == 2:
            pred = b
        elif f == 3:
            pred = (a + b) >> 1
        else:
            p = a + b - c
            pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
            pred = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
        out.append((x - pred) & 255)
    return bytes(out)


def _write_png_file(path, samples: np.ndarray, ctype: int, depth: int, interlace: bool, level: int, rng,
                    palette: np.ndarray | None = None):
    """samples: (H, W, channels) integers; every scanline gets a random filter."""
    h, w, ch = samples.shape
    bpp = max(1, ch * depth // 8)
    raw = bytearray()
    passes = _ADAM7 if interlace else ((0, 0, 1, 1),)
    for x0, y0, dx, dy in passes:
        sub = samples[y0::dy, x0::dx]
        if sub.size == 0:
            continue
        prev = bytes(len(_pack_row(sub[0].ravel(), depth)))
        for r in range(sub.shape[0]):
            row = _pack_row(sub[r].ravel(), depth)
            raw += _filter_row(row, prev, bpp, int(rng.integers(0, 5)))
            prev = row

    def chunk(t, body):
        return struct.pack(">I", len(body)) + t + body + struct.pack(">I", zlib.crc32(t + body) & 0xffffffff)
    data = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    data += chunk(b"tEXt", b"Comment\0made by the test")
    if palette is not None:
        data += chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    z = zlib.compress(bytes(raw), level)
    for k in range(0, len(z), 97):  # several IDAT chunks
        data += chunk(b"IDAT", z[k:k + 97])
    data += chunk(b"IEND", b"")
    path.write_bytes(data)


def _expected_rgb8(samples, ctype, depth, palette):
    if ctype == 3:
        return palette[samples[..., 0]].astype(np.uint8)
    s = samples.astype(np.uint32)
    s = s >> 8 if depth == 16 else s * {1: 255, 2: 0x55, 4: 0x11, 8: 1}[depth]
    if ctype in (0, 4):
        return np.repeat(s[..., :1], 3, axis=2).astype(np.uint8)
    return s[..., :3].astype(np.uint8)


def _png_cases():
    for ctype, depths in ((0, (1, 2, 4, 8, 16)), (2, (8, 16)), (3, (1, 2, 4, 8)), (4, (8, 16)), (6, (8, 16))):
        for depth in depths:
            yield ctype, depth


def test_png_load_every_colour_type_depth_and_filter(tmp_path):
    rng = np.random.default_rng(11)
    for ctype, depth in _png_cases():
        for (h, w), interlace, level in (((13, 21), False, 6), ((11, 17), True, 9), ((5, 3), True, 0),
                                         ((1, 1), False, 1)):
            ch = _CHANNELS[ctype]
            samples = rng.integers(0, 1 << depth, (h, w, ch))
            palette = None
            if ctype == 3:
                samples = samples % min(1 << depth, 40)
                palette = rng.integers(0, 256, (min(1 << depth, 40), 3))
            p = tmp_path / f"c{ctype}_d{depth}_{h}x{w}_{int(interlace)}.png"
            _write_png_file(p, samples, ctype, depth, interlace, level, rng, palette)
            want = _expected_rgb8(samples, ctype, depth, palette).astype(np.float32) / np.float32(255)
            got = N.load_image(p, flip_y=True)
            assert got.shape == (h, w, 3), (ctype, depth)
            assert np.array_equal(got, want), (ctype, depth, interlace, level)
            assert np.array_equal(N.load_image(p, flip_y=False), want[::-1])


def test_png_writer_reader_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, (70, 45, 3), dtype=np.uint8)
    p = tmp_path / "rt.png"
    N.write_png(p, img)
    assert np.array_equal(N.load_image(p, flip_y=True), img.astype(np.float32) / np.float32(255))


def test_png_load_errors(tmp_path):
    import pytest
    rng = np.random.default_rng(4)
    p = tmp_path / "ok.png"
    _write_png_file(p, rng.integers(0, 256, (9, 9, 3)), 2, 8, False, 6, rng)
    good = p.read_bytes()
    cases = {
        "crc": good[:40] + bytes([good[40] ^ 1]) + good[41:],
        "truncated": good[: len(good) // 2],
        "signature": b"\x89PNX" + good[4:],
    }
    for name, data in cases.items():
        q = tmp_path / f"{name}.png"
        q.write_bytes(data)
        with pytest.raises(N.PtError):
            N.load_image(q)


def test_png_texels_match_reference_image_texture(tmp_path):
    """PNG texels against the reference's ImageTexture (stbi_load /
    stbi_loadf) through the reference harness, where it is built: RGB 8- and
    16-bit, palette and Adam7 files (the three-component files the reference
    indexes correctly), LDR exact, isHDR within float rounding of powf."""
    import pytest
    from oracle.ref import refbind
    if not refbind.available():
        pytest.skip("reference harness not built")
    rng = np.random.default_rng(21)
    h, w = 16, 32
    xs, ys = np.meshgrid(np.arange(w - 1), np.arange(h - 1))
    uv = np.stack([xs.ravel() / w, ys.ravel() / h], 1).astype(np.float32)
    for ctype, depth, interlace in ((2, 8, False), (2, 16, False), (2, 8, True), (3, 4, False)):
        samples = rng.integers(0, 1 << depth, (h, w, _CHANNELS[ctype]))
        palette = rng.integers(0, 256, (16, 3)) if ctype == 3 else None
        p = tmp_path / f"ref_{ctype}_{depth}_{int(interlace)}.png"
        _write_png_file(p, samples, ctype, depth, interlace, 6, rng, palette)
        for flip in (False, True):
            ours = N.load_image(p, flip_y=flip)[ys.ravel(), xs.ravel()]
            assert np.array_equal(ours, refbind.image_texels(p, flip, False, uv)), (ctype, depth, flip)
            lin = N.load_image(p, flip_y=flip, hdr=True)[ys.ravel(), xs.ravel()]
            np.testing.assert_allclose(lin, refbind.image_texels(p, flip, True, uv), rtol=2e-7, atol=0)


def test_scene_image_texture_and_environment_from_files(tmp_path):
    from pathtracer_gb300 import scene as S
    rng = np.random.default_rng(8)
    png = tmp_path / "albedo.png"
    img = rng.integers(0, 256, (12, 20, 3), dtype=np.uint8)
    N.write_png(png, img)
    hdr = tmp_path / "sky.hdr"
    _write_hdr(hdr, _random_rgbe(rng, 16, 32), True)
    sc = S.Scene()
    t = sc.add_image_texture(png, flip_y=False)
    sc.set_environment(hdr, intensity=1.5)
    assert np.array_equal(sc.textures[t]["texels"], (img.astype(np.float32) / np.float32(255))[::-1])
    assert sc.env.shape == (16, 32, 3) and sc.env_intensity == 1.5
    assert np.array_equal(sc.env, N.load_image(hdr, hdr=True))


def test_reference_repository_pngs_decode_like_its_image_texture():
    """The reference repository's own PNGs (images/*.png: real-world files
    with dynamic Huffman blocks and every scanline filter) decoded here and
    sampled with ImageTexture's bilinear rule, against the reference's
    ImageTexture::getTexelColor on the same files through the harness."""
    import pytest
    from oracle.ref import refbind
    if not refbind.available() or refbind.REF_ROOT is None:
        pytest.skip("reference harness not built")
    files = sorted((refbind.REF_ROOT / "images").glob("*.png"))
    if not files:
        pytest.skip("reference images absent")
    rng = np.random.default_rng(17)
    uv = rng.uniform(0.0, 1.0, (2000, 2)).astype(np.float32)
    for f in files:
        for flip in (False, True):
            tex = N.load_image(f, flip_y=flip)  # [y][x]
            h, w, _ = tex.shape
            fu, fv = uv[:, 0] * np.float32(w), uv[:, 1] * np.float32(h)
            x = fu.astype(np.int64)
            y = fv.astype(np.int64)
            x1, y1 = fu - x, fv - y
            x = np.minimum(x, w - 2)
            y = np.minimum(y, h - 2)
            x2, y2 = np.float32(1) - x1, np.float32(1) - y1
            c12 = tex[y, x] * x2[:, None] + tex[y, x + 1] * x1[:, None]
            c34 = tex[y + 1, x] * x2[:, None] + tex[y + 1, x + 1] * x1[:, None]
            ours = c12 * y2[:, None] + c34 * y1[:, None]
            ref = refbind.image_texels(f, flip, False, uv)
            np.testing.assert_allclose(ours, ref, rtol=0, atol=2e-6, err_msg=f"{f.name} flip={flip}")


def test_oracle_blur_matches_reference_framebuffer():
    """The oracle's gaussianBlur restatement (which the GPU kernel matches
    bit for bit) against the reference's own FrameBuffer::gaussianBlur
    through the harness, where it is built."""
    import pytest
    from oracle.ref import refbind
    if not refbind.available():
        pytest.skip("reference harness not built")
    rng = np.random.default_rng(12)
    for (h, w), k, sigma in (((23, 31), 3, 1.0), ((40, 17), 5, 2.5), ((9, 9), 7, 0.8), ((64, 48), 11, 3.0)):
        img = rng.gamma(1.0, 1.0, (h, w, 3)).astype(np.float32)
        ours = O.gaussian_blur(img, k, sigma)
        ref = refbind.gaussian_blur(img, k, sigma)
        assert np.array_equal(ours, ref), (h, w, k, sigma, np.abs(ours - ref).max())


def test_tonemap_rule_matches_reference_fixture(golden):
    """The tone map rule pt_tonemap implements -- NaN -> 0, pow(v, 1/gamma),
    clamp to [0, 1], x 255 truncated, rows flipped (framebuffer.cpp:27-58) --
    restated in float32 reproduces the bytes the reference's writeToFile
    wrote (tests/golden/tonemap.npz)."""
    f = golden("tonemap.npz")["film"]
    for gamma in (2.2, 1.0):
        v = np.where(np.isnan(f), np.float32(0), np.power(f, np.float32(1.0) / np.float32(gamma)))
        b = (np.clip(v, 0, 1) * np.float32(255)).astype(np.uint8)[::-1]
        assert np.array_equal(b, golden("tonemap.npz")[f"rgb8_gamma_{gamma}"])
