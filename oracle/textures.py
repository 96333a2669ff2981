"""Oracle restatement of 2D textures (test infrastructure, not the product).

Texture2D nodes (builtin/btrc/builtin/texture2d/*, core/btrc/core/texture2d.h) compile to
postfix programs over an image table with the record layouts oracle.cpp reads (OTexImage,
OTexInstr, OMatTex). Images are decoded here with Python's zlib and our own PNG filter and
Radiance-HDR code (common/btrc/utils/image.cpp:296-346 semantics: 8-bit samples / 255, a
one-channel image reads (v, 0, 0, 1), sRGB decoding for 8-bit images when asked).
"""
from __future__ import annotations

import math
import struct
import zlib
from pathlib import Path

import numpy as np

IMG_DT = np.dtype([("offset", "<i4"), ("width", "<i4"), ("height", "<i4"), ("filter", "<i4"), ("au", "<i4"),
                   ("av", "<i4"), ("pad0", "<i4"), ("pad1", "<i4"), ("border", "<f4", 4)])
INSTR_DT = np.dtype([("op", "<i4"), ("image", "<i4"), ("a", "<f4", 6)])
MATTEX_DT = np.dtype([("prog", "<i4", 16), ("normal", "<i4"), ("pad", "<i4", 3)])
OP_END, OP_CONST, OP_SAMPLE, OP_ADD, OP_SUB, OP_MUL, OP_DIV = range(7)
ADDRESS = {"wrap": 0, "clamp": 1, "mirror": 2, "border": 3}


def f32(x):
    return np.float32(x)


# ---------------------------------------------------------------- image files

def _unfilter(raw: bytes, h: int, stride: int, bpp: int) -> np.ndarray:
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    pos = 0
    for y in range(h):
        ft = raw[pos]
        line = np.frombuffer(raw, np.uint8, stride, pos + 1).astype(np.int32)
        pos += stride + 1
        cur = np.zeros(stride, np.int32)
        if ft == 0:
            cur = line
        elif ft == 2:
            cur = (line + prev) & 255
        else:
            for x in range(stride):
                a = cur[x - bpp] if x >= bpp else 0
                b = prev[x]
                c = prev[x - bpp] if x >= bpp else 0
                if ft == 1:
                    p = a
                elif ft == 3:
                    p = (a + b) // 2
                elif ft == 4:
                    pp = a + b - c
                    pa, pb, pc = abs(pp - a), abs(pp - b), abs(pp - c)
                    p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                else:
                    raise ValueError("bad PNG filter")
                cur[x] = (line[x] + p) & 255
        out[y] = cur
        prev = cur
    return out


def load_png(path: str):
    data = Path(path).read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n", path
    pos, idat, plte, trns = 8, b"", b"", b""
    while pos + 12 <= len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if typ == b"IHDR":
            w, h, depth, ctype, _c, _f, inter = struct.unpack(">IIBBBBB", body[:13])
        elif typ == b"PLTE":
            plte = body
        elif typ == b"tRNS":
            trns = body
        elif typ == b"IDAT":
            idat += body
        elif typ == b"IEND":
            break
        pos += 12 + n
    if inter:
        raise ValueError("interlaced PNG")
    samples = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    raw = zlib.decompress(idat)
    stride = (w * samples * depth + 7) // 8
    bpp = max(1, samples * depth // 8)
    rows = _unfilter(raw, h, stride, bpp)
    if depth == 16:
        vals = rows.reshape(h, w * samples, 2)[..., 0].astype(np.int64)
    elif depth == 8:
        vals = rows.astype(np.int64)
    else:
        bits = np.unpackbits(rows, axis=1)[:, :w * samples * depth].reshape(h, w * samples, depth)
        vals = (bits * (1 << np.arange(depth - 1, -1, -1))).sum(-1)
        if ctype != 3:
            vals = vals * 255 // ((1 << depth) - 1)
    vals = vals.reshape(h, w, samples)
    rgba = np.zeros((h, w, 4), np.float32)
    rgba[..., 3] = 255
    if ctype == 3:
        pal = np.frombuffer(plte, np.uint8).reshape(-1, 3)
        idx = vals[..., 0]
        rgba[..., :3] = pal[idx]
        if trns:
            t = np.full(256, 255, np.int64)
            t[:len(trns)] = np.frombuffer(trns, np.uint8)
            rgba[..., 3] = t[idx]
        channels = 4 if trns else 3
    else:
        channels = samples
        if samples == 2:
            raise ValueError("ImageDynamic::load: unsupported channels: 2")
        rgba[..., :samples] = vals
    return rgba / f32(255), channels, False


def load_hdr(path: str):
    data = Path(path).read_bytes()
    pos = data.index(b"\n\n") + 2
    end = data.index(b"\n", pos)
    _ya, h, _xa, w = data[pos:end].split()
    h, w = int(h), int(w)
    pos = end + 1
    img = np.zeros((h, w, 4), np.float32)
    for y in range(h):
        if data[pos] == 2 and data[pos + 1] == 2 and 8 <= w < 32768:
            pos += 4
            scan = np.zeros((w, 4), np.uint8)
            for c in range(4):
                x = 0
                while x < w:
                    cnt = data[pos]
                    pos += 1
                    if cnt > 128:
                        scan[x:x + cnt - 128, c] = data[pos]
                        pos += 1
                        x += cnt - 128
                    else:
                        scan[x:x + cnt, c] = np.frombuffer(data, np.uint8, cnt, pos)
                        pos += cnt
                        x += cnt
        else:
            scan = np.frombuffer(data, np.uint8, w * 4, pos).reshape(w, 4)
            pos += w * 4
        e = scan[:, 3].astype(np.int64)
        f = np.where(e > 0, np.ldexp(np.float32(1), (e - 136).astype(np.int32)).astype(np.float32), f32(0))
        img[y, :, :3] = scan[:, :3].astype(np.float32) * f[:, None]
        img[y, :, 3] = 1
    return img, 3, True


def load_image(path: str):
    ext = Path(path).suffix.lower()
    if ext == ".png":
        return load_png(path)
    if ext == ".hdr":
        return load_hdr(path)
    raise ValueError("unsupported image format " + ext)


# ---------------------------------------------------------------- texture programs

class TexStore:
    def __init__(self, sdir: str):
        self.sdir = sdir
        self.images: list[tuple] = []
        self.texels: list[np.ndarray] = []
        self.ntexel = 0
        self.instr: list[tuple] = []
        self.cache: dict = {}

    def _image(self, n, vvec3, vfloat) -> int:
        fn = n.child("filename").s.replace("$env{scene_directory}", self.sdir)
        au = ADDRESS[n.child("address_mode_u").s] if n.find("address_mode_u") is not None else 1
        av = ADDRESS[n.child("address_mode_v").s] if n.find("address_mode_v") is not None else 1
        filt = n.child("filter").s if n.find("filter") is not None else "linear"
        srgb = n.find("srgb_to_linear") is not None and n.child("srgb_to_linear").s == "true"
        border = [0.0, 0.0, 0.0, 0.0]
        if n.find("border") is not None:
            b = n.child("border")
            if b.kind == "array" and len(b.elems) == 3:
                border[:3] = [float(vfloat(e)) for e in b.elems]
            else:
                v = float(vfloat(b.elems[0] if b.kind == "array" else b))
                border = [v] * 4
        key = (fn, au, av, filt, srgb, tuple(border))
        if key in self.cache:
            return self.cache[key]
        img, _ch, is_float = load_image(fn)
        if srgb and not is_float:
            c = img[..., :3]
            img[..., :3] = np.where(c <= f32(0.04045), c / f32(12.92),
                                    np.power((c + f32(0.055)) / f32(1.055), f32(2.4))).astype(np.float32)
        h, w = img.shape[:2]
        self.images.append((self.ntexel, w, h, 0 if filt == "point" else 1, au, av, 0, 0, border))
        self.texels.append(img.reshape(-1, 4).astype(np.float32))
        self.ntexel += w * h
        self.cache[key] = len(self.images) - 1
        return self.cache[key]

    def compile(self, n, vvec3, vfloat, parse_t2):
        """Returns (constant rgb, None) or (None, first instruction)."""
        const = self._const(n, vvec3)
        if const is not None:
            return const, None
        code: list[tuple] = []
        self._emit(n, np.array([[1, 0, 0], [0, 1, 0]], np.float32), code, vvec3, vfloat, parse_t2)
        code.append((OP_END, 0, [0] * 6))
        start = len(self.instr)
        self.instr.extend(code)
        return None, start

    def constant_program(self, rgb) -> int:
        start = len(self.instr)
        self.instr.append((OP_CONST, 0, [float(rgb[0]), float(rgb[1]), float(rgb[2]), 0, 0, 0]))
        self.instr.append((OP_END, 0, [0] * 6))
        return start

    @staticmethod
    def _const(n, vvec3):
        if n.kind in ("value", "array"):
            return vvec3(n)
        if n.child("type").s == "constant":
            return vvec3(n.child("value"))
        return None

    def _emit(self, n, m, code, vvec3, vfloat, parse_t2):
        c = self._const(n, vvec3)
        if c is not None:
            code.append((OP_CONST, 0, [float(c[0]), float(c[1]), float(c[2]), 0, 0, 0]))
            return
        t = n.child("type").s
        if t == "array":
            code.append((OP_SAMPLE, self._image(n, vvec3, vfloat), [float(v) for v in m.reshape(-1)]))
        elif t in ("add", "sub", "mul", "div"):
            self._emit(n.child("lhs"), m, code, vvec3, vfloat, parse_t2)
            self._emit(n.child("rhs"), m, code, vvec3, vfloat, parse_t2)
            code.append(({"add": OP_ADD, "sub": OP_SUB, "mul": OP_MUL, "div": OP_DIV}[t], 0, [0] * 6))
        elif t == "transform":
            tm = parse_t2(n.child("transform"))
            self._emit(n.child("tex"), _affine_mul(tm, m), code, vvec3, vfloat, parse_t2)
        else:
            raise ValueError("texture2d type " + t)

    def arrays(self):
        imgs = np.zeros(max(1, len(self.images)), IMG_DT)
        for i, r in enumerate(self.images):
            imgs[i] = r
        tex = np.ascontiguousarray(np.concatenate(self.texels) if self.texels else np.zeros((1, 4), np.float32))
        ins = np.zeros(max(1, len(self.instr)), INSTR_DT)
        for i, r in enumerate(self.instr):
            ins[i] = r
        return imgs, tex, ins


def _affine_mul(x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """3x3 product of two affine maps (rows of 2x3), float32 in the reference's order."""
    X = np.vstack([x, [0, 0, 1]]).astype(np.float32)
    Y = np.vstack([y, [0, 0, 1]]).astype(np.float32)
    r = np.zeros((2, 3), np.float32)
    for i in range(2):
        for j in range(3):
            s = f32(0)
            for k in range(3):
                s = f32(s + f32(X[i, k] * Y[k, j]))
            r[i, j] = s
    return r


def parse_transform2d(n, vfloat, vradian) -> np.ndarray:
    """parse_transform2d (factory/btrc/factory/node/node.cpp:126-164) as a 2x3 map."""
    ident = np.array([[1, 0, 0], [0, 1, 0]], np.float32)
    if n.kind == "array":
        t = ident
        for e in n.elems:
            t = _affine_mul(parse_transform2d(e, vfloat, vradian), t)
        return t

    def vec2(c):
        if c.kind == "array":
            return (float(vfloat(c.elems[0])), float(vfloat(c.elems[0 if len(c.elems) == 1 else 1])))
        v = float(vfloat(c))
        return v, v
    if n.find("translate") is not None:
        x, y = vec2(n.child("translate"))
        return np.array([[1, 0, x], [0, 1, y]], np.float32)
    if n.find("rotate") is not None:
        r = float(vradian(n.child("rotate").child("angle")))
        s, c = f32(math.sin(f32(r))), f32(math.cos(f32(r)))
        return np.array([[c, -s, 0], [s, c, 0]], np.float32)
    if n.find("scale") is not None:
        x, y = vec2(n.child("scale"))
        return np.array([[x, 0, 0], [0, y, 0]], np.float32)
    for key, m in (("inverse_u", [[-1, 0, 1], [0, 1, 0]]), ("inverse_v", [[1, 0, 0], [0, -1, 1]]),
                   ("swap_uv", [[0, 1, 0], [1, 0, 0]])):
        if n.find(key) is not None and n.child(key).s == "true":
            return np.array(m, np.float32)
    raise ValueError("unknown transform2d type")
