"""Image files of the `save` post-processor (btrc_image_save), read back with minimal
decoders written here from the format specifications:

  * PNG: 8-bit RGBA, byte = min(int(v * 256), 255) of the gamma-corrected value and
    alpha 255 (common/btrc/utils/image.h:207-217, save_to_image.cpp:30-43);
  * OpenEXR: float B, G, R scanlines (common/btrc/utils/image.cpp:51-110);
  * Radiance HDR: RGBE;
  * JPEG: BTRC_ERR_UNSUPPORTED; an unknown extension: BTRC_ERR_INVALID_ARG."""
import struct
import zlib

import numpy as np
import pytest

import btrc_gb300 as B


@pytest.fixture(scope="module")
def host_ctx(native_lib):
    ctx = B.Context(-1)
    yield ctx
    ctx.close()


def read_png(path):
    data = path.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat = 8, b""
    w = h = None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xffffffff
        if typ == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8 and ctype == 6
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 4 * w)
    assert (rows[:, 0] == 0).all()
    return rows[:, 1:].reshape(h, w, 4)


def read_exr(path):
    data = path.read_bytes()
    magic, version = struct.unpack("<II", data[:8])
    assert magic == 20000630 and version == 2
    pos, attrs = 8, {}
    while data[pos] != 0:
        e = data.index(b"\0", pos)
        name = data[pos:e].decode()
        e2 = data.index(b"\0", e + 1)
        typ = data[e + 1:e2].decode()
        size, = struct.unpack("<i", data[e2 + 1:e2 + 5])
        attrs[name] = (typ, data[e2 + 5:e2 + 5 + size])
        pos = e2 + 5 + size
    pos += 1
    assert attrs["compression"][1] == b"\0"
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    chl = attrs["channels"][1]
    names, p = [], 0
    while chl[p] != 0:
        e = chl.index(b"\0", p)
        names.append(chl[p:e].decode())
        assert struct.unpack("<i", chl[e + 1:e + 5])[0] == 2  # FLOAT
        p = e + 1 + 16
    offsets = struct.unpack(f"<{h}Q", data[pos:pos + 8 * h])
    img = np.zeros((h, w, len(names)), np.float32)
    for y in range(h):
        o = offsets[y]
        ly, n = struct.unpack("<ii", data[o:o + 8])
        assert n == 4 * w * len(names)
        img[ly] = np.frombuffer(data[o + 8:o + 8 + n], np.float32).reshape(len(names), w).T
    return {c: img[..., k] for k, c in enumerate(names)}


def read_hdr(path):
    data = path.read_bytes()
    head_end = data.index(b"\n\n") + 2
    line_end = data.index(b"\n", head_end)
    _, h, _, w = data[head_end:line_end].split()
    h, w = int(h), int(w)
    px = np.frombuffer(data[line_end + 1:], np.uint8).reshape(h, w, 4).astype(np.float64)
    e = px[..., 3:4]
    return np.where(e > 0, px[..., :3] * np.ldexp(1.0, (e - 136).astype(int)), 0.0)


def _image(rng, h=7, w=11):
    return rng.uniform(-0.2, 1.3, (h, w, 3)).astype(np.float32)


def test_png_bytes_follow_reference_rule(host_ctx, tmp_path):
    img = _image(np.random.default_rng(1))
    img[0, 0] = [0.999, 1.0, 0.00390625]
    p = tmp_path / "a.png"
    host_ctx.image_save(p, img, gamma=2.2)
    got = read_png(p)
    with np.errstate(invalid="ignore"):
        g = np.power(img.astype(np.float32), np.float32(1 / 2.2))
    finite = np.isfinite(g)
    want = np.minimum((np.where(finite, g, 0) * 256).astype(np.int64), 255)
    assert (got[..., 3] == 255).all()
    assert np.array_equal(got[..., :3][finite], (want[finite] & 0xff).astype(np.uint8))
    # pow of a negative base is NaN, which converts to byte 0
    assert (got[..., :3][~finite] == 0).all()
    # negative values without gamma wrap modulo 256
    p2 = tmp_path / "neg.png"
    host_ctx.image_save(p2, np.full((1, 1, 3), -0.5, np.float32))
    assert (read_png(p2)[0, 0, :3] == 128).all()
    assert got[0, 0, 1] == 255 and got[0, 0, 0] == 255 and got[0, 0, 2] == int(0.00390625 ** (1 / 2.2) * 256)


def test_png_four_channels(host_ctx, tmp_path):
    img = np.random.default_rng(2).uniform(0, 1, (5, 4, 4)).astype(np.float32)
    p = tmp_path / "b.PNG"
    host_ctx.image_save(p, img)
    got = read_png(p)
    assert np.array_equal(got, np.minimum((img * 256).astype(np.int64), 255).astype(np.uint8))


def test_exr_float_channels(host_ctx, tmp_path):
    img = _image(np.random.default_rng(3), 9, 6)
    p = tmp_path / "c.exr"
    host_ctx.image_save(p, img)
    ch = read_exr(p)
    assert sorted(ch) == ["B", "G", "R"]
    assert np.array_equal(ch["R"], img[..., 0]) and np.array_equal(ch["G"], img[..., 1])
    assert np.array_equal(ch["B"], img[..., 2])


def test_hdr_rgbe(host_ctx, tmp_path):
    img = np.abs(_image(np.random.default_rng(4))) * 20
    p = tmp_path / "d.hdr"
    host_ctx.image_save(p, img)
    got = read_hdr(p)
    # RGBE keeps 8 mantissa bits of the largest component: error below max / 128
    tol = img.max(-1, keepdims=True) / 128.0
    assert (np.abs(got - img) <= tol + 1e-6).all()


def test_unsupported_and_bad_extension(host_ctx, tmp_path):
    img = np.zeros((2, 2, 3), np.float32)
    with pytest.raises(B.BtrcError) as e:
        host_ctx.image_save(tmp_path / "e.jpg", img)
    assert e.value.status == 8  # UNSUPPORTED
    with pytest.raises(B.BtrcError) as e:
        host_ctx.image_save(tmp_path / "e.bmp", img)
    assert e.value.status == 1  # INVALID_ARG
    with pytest.raises(B.BtrcError) as e:
        host_ctx.image_save(tmp_path / "no_such_dir" / "e.png", img)
    assert e.value.status == 2  # IO


def test_texture_decoders_match_oracle(host_ctx, tmp_path):
    # PNG: every filter type, 8/16/4-bit grey, RGB, RGBA, palette + tRNS; HDR: RLE scanlines
    from btrc_gb300 import scenes
    from oracle import textures as OT
    rng = np.random.default_rng(11)
    cases = {
        "rgb.png": dict(img=rng.integers(0, 256, (13, 17, 3))),
        "rgba.png": dict(img=rng.integers(0, 256, (9, 21, 4))),
        "g8.png": dict(img=rng.integers(0, 256, (7, 9))),
        "g16.png": dict(img=rng.integers(0, 65536, (11, 5)), depth=16),
        "g4.png": dict(img=rng.integers(0, 16, (6, 13)), depth=4),
        "g1.png": dict(img=rng.integers(0, 2, (5, 19)), depth=1),
        "pal.png": dict(img=rng.integers(0, 6, (8, 8)), palette=rng.integers(0, 256, (6, 3)), alpha=[255, 0, 77]),
    }
    for name, kw in cases.items():
        scenes.write_png(tmp_path / name, **kw)
        got, ch = host_ctx.image_load(tmp_path / name)
        want, wch, _ = OT.load_png(str(tmp_path / name))
        assert ch == wch, name
        assert np.array_equal(got, want), name
    sky = rng.uniform(0, 5, (9, 40, 3)) * (rng.random((9, 40, 1)) < 0.7)
    sky[:, 10:30] = 2.5  # long runs
    scenes.write_hdr(tmp_path / "s.hdr", sky)
    got, ch = host_ctx.image_load(tmp_path / "s.hdr")
    want, _, _ = OT.load_hdr(str(tmp_path / "s.hdr"))
    assert ch == 3 and np.array_equal(got, want)
    assert np.allclose(got[..., :3], sky, rtol=1 / 64, atol=1e-6 + sky.max(-1, keepdims=True) / 128)
    with pytest.raises(B.BtrcError) as e:
        host_ctx.image_load(tmp_path / "x.jpg")
    assert e.value.status == 8
