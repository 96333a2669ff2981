"""ORACLE — test infrastructure only. Python restatement of the reference's scene
assembly, independent of the product's C++ loader:

  * JSON with "$include{}" splicing and "$reference{}" resolution and every scalar kept as
    the string std::to_string would make (factory/btrc/factory/node/parser.cpp:16-72,106-…);
  * transforms as (mat, inv) pairs composed in FP32 (factory/btrc/factory/node/node.cpp:166-214,
    common/btrc/utils/math/{mat4,transform}.cpp);
  * OBJ triangles and per-triangle shading records
    (common/btrc/utils/triangle_mesh_loader.cpp:16-150, builtin/.../geometry/triangle_mesh.cpp:24-171);
  * entities, materials, area lights, sky (factory/btrc/factory/scene.cpp:5-94);
  * pinhole camera (builtin/btrc/builtin/camera/pinhole.cpp:55-77).

The result feeds oracle.cpp through the OracleScene structure.
"""
from __future__ import annotations

import json
import math
import os
import re
from pathlib import Path

import numpy as np

from . import OracleScene, _p, lib
from .textures import MATTEX_DT, TexStore, parse_transform2d

f32 = np.float32


# ------------------------------------------------------------------ JSON with Btrc semantics

class Node:
    __slots__ = ("kind", "members", "elems", "s")

    def __init__(self, kind, members=None, elems=None, s=None):
        self.kind, self.members, self.elems, self.s = kind, members, elems, s

    def find(self, key):
        if self.kind != "group":
            return None
        for k, v in self.members:
            if k == key:
                return v
        return None

    def child(self, key):
        v = self.find(key)
        if v is None:
            raise KeyError(key)
        return v


def _to_string_float(x: float) -> str:
    # std::to_string(float): "%f" of the float widened to double
    return "%f" % float(f32(x))


def _strip_comments(text: str) -> str:
    out, i, n, in_str = [], 0, len(text), False
    while i < n:
        c = text[i]
        if in_str:
            out.append(c)
            if c == "\\" and i + 1 < n:
                out.append(text[i + 1])
                i += 2
                continue
            if c == '"':
                in_str = False
            i += 1
            continue
        if c == '"':
            in_str = True
            out.append(c)
            i += 1
        elif text.startswith("//", i):
            j = text.find("\n", i)
            i = n if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            i = n if j < 0 else j + 2
        else:
            out.append(c)
            i += 1
    return "".join(out)


def _to_node(v) -> Node:
    if isinstance(v, dict):
        return Node("group", members=[(k, _to_node(x)) for k, x in v.items()])
    if isinstance(v, list):
        return Node("array", elems=[_to_node(x) for x in v])
    if isinstance(v, bool):
        return Node("value", s="true" if v else "false")
    if isinstance(v, int):
        return Node("value", s=str(int(np.int32(v))))
    if isinstance(v, float):
        return Node("value", s=_to_string_float(v))
    if v is None:
        return Node("value", s="")
    return Node("value", s=str(v))


def _find_ref(path: list[Node], ref: str) -> Node:
    secs = [s for s in ref.split("/") if s]
    if secs[0] == "$root":
        start = 0
    else:
        start = -1
        for k in range(len(path) - 1, -1, -1):
            n = path[k]
            if n.kind == "group" and n.find(secs[0]) is not None:
                start = k
                break
            if n.kind == "array" and secs[0].isdigit() and int(secs[0]) < len(n.elems):
                start = k
                break
        if start < 0:
            raise KeyError(ref)
    node = path[start]
    for i, s in enumerate(secs):
        if i == 0 and s == "$root":
            continue
        node = node.child(s) if node.kind == "group" else node.elems[int(s)]
    return node


def _resolve(path: list[Node], holder, key):
    node = holder[key]
    if node.kind == "group":
        path.append(node)
        for idx in range(len(node.members)):
            k, _ = node.members[idx]
            box = [node.members[idx][1]]
            _resolve(path, box, 0)
            node.members[idx] = (k, box[0])
        path.pop()
    elif node.kind == "array":
        path.append(node)
        for idx in range(len(node.elems)):
            _resolve(path, node.elems, idx)
        path.pop()
    elif node.s.startswith("$reference{"):
        holder[key] = _find_ref(path, node.s[11:-1])


def parse_scene_json(path: str | os.PathLike) -> tuple[Node, str]:
    path = Path(path)
    scene_dir = str(path.resolve().parent)
    src = path.read_text()
    while True:
        b = src.find('"$include{')
        if b < 0:
            break
        e = src.find('}"', b + 10)
        inc = Path(src[b + 10:e])
        if not inc.is_absolute():
            inc = Path(scene_dir) / inc
        src = src[:b] + inc.read_text() + src[e + 2:]
    root = _to_node(json.loads(_strip_comments(src)))
    box = [root]
    path_nodes = [root]
    for idx in range(len(root.members)):
        k, _ = root.members[idx]
        holder = [root.members[idx][1]]
        _resolve(path_nodes, holder, 0)
        root.members[idx] = (k, holder[0])
    return box[0], scene_dir


def vfloat(n: Node) -> np.float32:
    return f32(float(n.s))  # std::stof


def vvec3(n: Node) -> np.ndarray:
    if n.kind == "array":
        if len(n.elems) == 1:
            return np.array([vfloat(n.elems[0])] * 3, np.float32)
        return np.array([vfloat(e) for e in n.elems], np.float32)
    return np.array([vfloat(n)] * 3, np.float32)


def vangle_rad(n: Node) -> np.float32:
    if n.find("deg") is not None:
        return f32(f32(math.pi) / f32(180.0)) * vfloat(n.find("deg"))
    return vfloat(n.find("rad"))


def vangle_deg(n: Node) -> np.float32:
    if n.find("deg") is not None:
        return vfloat(n.find("deg"))
    return f32(f32(180.0) / f32(math.pi)) * vfloat(n.find("rad"))


# ------------------------------------------------------------------ transforms (FP32, reference op order)

def mat_rows(*v) -> np.ndarray:
    return np.array(v, np.float32).reshape(4, 4)


def mat_mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    r = np.zeros((4, 4), np.float32)
    for i in range(4):
        for j in range(4):
            s = a[i, 0] * b[0, j]
            s = f32(s + a[i, 1] * b[1, j])
            s = f32(s + a[i, 2] * b[2, j])
            s = f32(s + a[i, 3] * b[3, j])
            r[i, j] = s
    return r


def _rot_axis(axis: np.ndarray, rad) -> np.ndarray:
    a = axis / f32(np.sqrt(f32(np.dot(axis, axis))))
    a = a.astype(np.float32)
    s, c = f32(np.sin(f32(rad))), f32(np.cos(f32(rad)))
    one = f32(1)
    R = [[a[0] * a[0] + (one - a[0] * a[0]) * c, a[0] * a[1] * (one - c) - a[2] * s, a[0] * a[2] * (one - c) + a[1] * s],
         [a[0] * a[1] * (one - c) + a[2] * s, a[1] * a[1] + (one - a[1] * a[1]) * c, a[1] * a[2] * (one - c) - a[0] * s],
         [a[0] * a[2] * (one - c) - a[1] * s, a[1] * a[2] * (one - c) + a[0] * s, a[2] * a[2] + (one - a[2] * a[2]) * c]]
    # stored transposed (the reference writes the textbook entries into column-major storage)
    return mat_rows(R[0][0], R[1][0], R[2][0], 0, R[0][1], R[1][1], R[2][1], 0, R[0][2], R[1][2], R[2][2], 0,
                    0, 0, 0, 1)


def parse_transform(n: Node) -> tuple[np.ndarray, np.ndarray]:
    I = np.eye(4, dtype=np.float32)
    if n.kind == "array":
        mat, inv = I.copy(), I.copy()
        for e in n.elems:
            m2, i2 = parse_transform(e)
            mat, inv = mat_mul(m2, mat), mat_mul(inv, i2)
        return mat, inv
    if n.find("translate") is not None:
        t = vvec3(n.find("translate"))
        return (mat_rows(1, 0, 0, t[0], 0, 1, 0, t[1], 0, 0, 1, t[2], 0, 0, 0, 1),
                mat_rows(1, 0, 0, -t[0], 0, 1, 0, -t[1], 0, 0, 1, -t[2], 0, 0, 0, 1))
    if n.find("rotate") is not None:
        r = n.find("rotate")
        axis, rad = vvec3(r.child("axis")), vangle_rad(r.child("angle"))
        return _rot_axis(axis, rad), _rot_axis(axis, -rad)
    for key in ("rotate_x", "rotate_y", "rotate_z"):
        if n.find(key) is not None:
            rad = vangle_rad(n.find(key))

            def rm(r):
                S, C = f32(np.sin(f32(r))), f32(np.cos(f32(r)))
                if key == "rotate_x":
                    return mat_rows(1, 0, 0, 0, 0, C, -S, 0, 0, S, C, 0, 0, 0, 0, 1)
                if key == "rotate_y":
                    return mat_rows(C, 0, S, 0, 0, 1, 0, 0, -S, 0, C, 0, 0, 0, 0, 1)
                return mat_rows(C, -S, 0, 0, S, C, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1)

            if key == "rotate_z":
                return rm(-rad), rm(-rad)
            return rm(rad), rm(-rad)
    if n.find("scale") is not None:
        s = vvec3(n.find("scale"))
        one = f32(1)
        return (mat_rows(s[0], 0, 0, 0, 0, s[1], 0, 0, 0, 0, s[2], 0, 0, 0, 0, 1),
                mat_rows(one / s[0], 0, 0, 0, 0, one / s[1], 0, 0, 0, 0, one / s[2], 0, 0, 0, 0, 1))
    raise ValueError("unknown transform3d type")


def apply_point(m: np.ndarray, p: np.ndarray) -> np.ndarray:
    """Rows of (N, 3) float32 points through the 3x4 part, left-to-right FP32 sums."""
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    cols = []
    for r in range(3):
        v = m[r, 0] * x
        v = (v + m[r, 1] * y).astype(np.float32)
        v = (v + m[r, 2] * z).astype(np.float32)
        v = (v + m[r, 3]).astype(np.float32)
        cols.append(v)
    return np.stack(cols, axis=1).astype(np.float32)


# ------------------------------------------------------------------ OBJ + per-triangle data

def _nrm(v: np.ndarray) -> np.ndarray:
    l = np.sqrt((v * v).sum(-1, dtype=np.float32)).astype(np.float32)
    return (v * (f32(1) / l)[..., None]).astype(np.float32)


def _cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                     a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], -1).astype(np.float32)


def _obj_fast(text: str):
    """Vectorised parse for OBJ files whose faces are all triangles in one index format
    (v, v/t, v//n or v/t/n). Returns None when the file needs the general parser."""
    lines = text.split("\n")
    vl = [l[2:] for l in lines if l.startswith("v ")]
    nl = [l[3:] for l in lines if l.startswith("vn ")]
    tl = [l[3:] for l in lines if l.startswith("vt ")]
    fl = [l[2:] for l in lines if l.startswith("f ")]
    if not fl:
        return None
    first = fl[0].split()
    if len(first) != 3:
        return None
    tok = first[0]
    slashes = tok.count("/")
    fmt = "v" if slashes == 0 else ("vn" if "//" in tok else ("vt" if slashes == 1 else "vtn"))
    per = {"v": 1, "vt": 2, "vn": 2, "vtn": 3}[fmt]
    body = " ".join(fl).replace("//", " ").replace("/", " ")
    ints = np.array(body.split(), dtype=np.int64)
    if len(ints) != len(fl) * 3 * per:
        return None
    ints = ints.reshape(-1, 3, per)
    V = np.array(" ".join(vl).split(), dtype=np.float64).astype(np.float32).reshape(-1, 3)
    N = np.array(" ".join(nl).split(), dtype=np.float64).astype(np.float32).reshape(-1, 3) if nl else np.zeros((0, 3), np.float32)
    T = np.array(" ".join(tl).split(), dtype=np.float64).astype(np.float32).reshape(-1, 3)[:, :2] if False else (
        np.array([[float(x) for x in l.split()[:2]] for l in tl], np.float32).reshape(-1, 2) if tl else np.zeros((0, 2), np.float32))
    F = np.full((len(fl), 3, 3), 0, np.int64)

    def res(i, n):
        return np.where(i > 0, i - 1, np.where(i < 0, n + i, -1))

    F[:, :, 0] = res(ints[:, :, 0], len(V))
    F[:, :, 1] = res(ints[:, :, 1], len(T)) if fmt in ("vt", "vtn") else -1
    F[:, :, 2] = res(ints[:, :, {"vn": 1, "vtn": 2}[fmt]], len(N)) if fmt in ("vn", "vtn") else -1
    return V, N, T, F


def load_obj(path: str, to_unit_cube: bool):
    text = Path(path).read_text()
    fast = _obj_fast(text)
    if fast is not None:
        V, N, T, F = fast
        return _obj_records(V, N, T, F, to_unit_cube)
    V, N, T, faces = [], [], [], []
    for line in text.split("\n"):
        if line.startswith("v "):
            V.append([float(t) for t in line.split()[1:4]])
        elif line.startswith("vn "):
            N.append([float(t) for t in line.split()[1:4]])
        elif line.startswith("vt "):
            T.append([float(t) for t in line.split()[1:3]])
        elif line.startswith("f "):
            cs = []
            for tok in line.split()[1:]:
                parts = tok.split("/")
                vi = int(parts[0])
                ti = int(parts[1]) if len(parts) > 1 and parts[1] else 0
                ni = int(parts[2]) if len(parts) > 2 and parts[2] else 0
                cs.append((vi, ti, ni))
            for k in range(1, len(cs) - 1):
                faces.append((cs[0], cs[k], cs[k + 1]))
    V = np.array(V, np.float32).reshape(-1, 3)
    N = np.array(N, np.float32).reshape(-1, 3)
    T = np.array(T, np.float32).reshape(-1, 2)

    def res(i, n):
        return i - 1 if i > 0 else (n + i if i < 0 else -1)

    F = np.array([[[res(c[0], len(V)), res(c[1], len(T)), res(c[2], len(N))] for c in f] for f in faces],
                 np.int64).reshape(-1, 3, 3)
    return _obj_records(V, N, T, F, to_unit_cube)


def procedural(kind: str, subdivisions: int = 3):
    """Inline geometry creators of the scene format extension: "sphere" (icosphere of
    radius 1 with `subdivisions` levels, smooth normals, spherical texture coordinates),
    "quad" (unit square in xz facing +y, uv over [0,1]^2), "box" ([-0.5, 0.5]^3 facing
    outwards, flat); built in float64 and rounded once, like the loader."""
    if kind == "sphere":
        t = (1.0 + math.sqrt(5.0)) / 2.0
        v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
        verts = [np.array(q, np.float64) / math.sqrt(sum(x * x for x in q)) for q in v]
        faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
                 (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
                 (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
        for _ in range(subdivisions):
            cache = {}

            def mid(a, b):
                key = (min(a, b), max(a, b))
                if key not in cache:
                    m = verts[a] + verts[b]
                    verts.append(m / math.sqrt(float(m @ m)))
                    cache[key] = len(verts) - 1
                return cache[key]
            nf = []
            for a, b, c in faces:
                ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
                nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
            faces = nf
        P = np.array(verts, np.float64)
        V = P.astype(np.float32)
        T = np.stack([np.arctan2(P[:, 2], P[:, 0]) / (2 * math.pi) + 0.5,
                      np.arccos(np.clip(P[:, 1], -1, 1)) / math.pi], 1).astype(np.float32)
        f = np.array(faces, np.int64)
        F = np.stack([f, f, f], -1)
        return _obj_records(V, V.copy(), T, F, False)
    if kind == "quad":
        V = np.array([[-0.5, 0, -0.5], [0.5, 0, -0.5], [0.5, 0, 0.5], [-0.5, 0, 0.5]], np.float32)
        T = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
        f = np.array([[0, 2, 1], [0, 3, 2]], np.int64)
        F = np.stack([f, f, np.full_like(f, -1)], -1)
        return _obj_records(V, np.zeros((0, 3), np.float32), T, F, False)
    if kind == "box":
        V = np.array([[0.5 if c & 4 else -0.5, 0.5 if c & 2 else -0.5, 0.5 if c & 1 else -0.5] for c in range(8)],
                     np.float32)
        f = np.array([[0, 1, 3], [0, 3, 2], [4, 6, 7], [4, 7, 5], [0, 4, 5], [0, 5, 1], [2, 3, 7], [2, 7, 6],
                      [0, 2, 6], [0, 6, 4], [1, 5, 7], [1, 7, 3]], np.int64)
        F = np.stack([f, np.full_like(f, -1), np.full_like(f, -1)], -1)
        return _obj_records(V, np.zeros((0, 3), np.float32), np.zeros((0, 2), np.float32), F, False)
    raise ValueError("geometry type " + kind)


def _obj_records(V, N, T, F, to_unit_cube):
    if to_unit_cube and len(V):
        lo, hi = V.min(0), V.max(0)
        ext = (hi - lo).astype(np.float32)
        emax = ext.max()
        s = f32(1) / emax if emax > 0 else f32(1)
        V = (s * (V - f32(0.5) * (lo + hi))).astype(np.float32)
    a, b, c = V[F[:, 0, 0]], V[F[:, 1, 0]], V[F[:, 2, 0]]
    geo_z = _nrm(_cross(b - a, c - a))
    sz = []
    uv = []
    for k in range(3):
        ni = F[:, k, 2]
        nk = geo_z.copy()
        if len(N):
            nk = np.where((ni >= 0)[:, None], N[np.maximum(ni, 0)], geo_z).astype(np.float32)
        zero = (nk == 0).all(-1)
        nk[zero] = geo_z[zero]
        sz.append(nk)
        ti = F[:, k, 1]
        uvk = np.zeros((len(F), 2), np.float32)
        if len(T):
            uvk = np.where((ti >= 0)[:, None], T[np.maximum(ti, 0)], uvk).astype(np.float32)
        uv.append(uvk)
    # triangle_dpdu (common/btrc/utils/math/triangle.h)
    ba, ca = (b - a).astype(np.float32), (c - a).astype(np.float32)
    m00, m01 = uv[1][:, 0] - uv[0][:, 0], uv[1][:, 1] - uv[0][:, 1]
    m10, m11 = uv[2][:, 0] - uv[0][:, 0], uv[2][:, 1] - uv[0][:, 1]
    det = (m00 * m11 - m01 * m10).astype(np.float32)
    gx = np.zeros_like(a)
    nz = det != 0
    if nz.any():
        inv = (f32(1) / det[nz]).astype(np.float32)
        gx[nz] = _nrm(((m11[nz] * inv)[:, None] * ba[nz] - (m01[nz] * inv)[:, None] * ca[nz]).astype(np.float32))
    if (~nz).any():
        z = _nrm(geo_z[~nz])
        y = np.where((f32(1) - np.abs(z[:, 0]) < f32(0.1))[:, None],
                     _cross(z, np.array([0, 1, 0], np.float32)), _cross(z, np.array([1, 0, 0], np.float32)))
        # Frame::from_z(nor).x = z cross y (common/btrc/utils/math/frame.cpp:45-57)
        gx[~nz] = _nrm(_cross(z, y))
    gy = _nrm(_cross(geo_z, gx))
    shade = np.zeros((6, len(F), 4), np.float32)
    shade[0, :, :3], shade[0, :, 3] = gx, uv[0][:, 0]
    shade[1, :, :3], shade[1, :, 3] = gy, uv[1][:, 0] - uv[0][:, 0]
    shade[2, :, :3], shade[2, :, 3] = geo_z, uv[2][:, 0] - uv[0][:, 0]
    shade[3, :, :3], shade[3, :, 3] = sz[0], uv[0][:, 1]
    shade[4, :, :3], shade[4, :, 3] = sz[1] - sz[0], uv[1][:, 1] - uv[0][:, 1]
    shade[5, :, :3], shade[5, :, 3] = sz[2] - sz[0], uv[2][:, 1] - uv[0][:, 1]
    cr = _cross(ba, ca)
    area = (f32(0.5) * np.sqrt((cr * cr).sum(-1, dtype=np.float32))).astype(np.float32)
    pos = np.stack([a, b, c], 1).astype(np.float32)
    return pos, shade, area


# ------------------------------------------------------------------ full scene

MAT_TYPES = {"diffuse": 0, "metal": 1, "disney": 2, "black": 3, "invisible": 4, "mirror": 5, "glass": 6}


def _material(n: Node, T: TexStore):
    """Material record (20 floats: type, shadow terminator, p[16], pad) and, when a
    parameter is a non-constant Texture2D or a normal map is present, its MaterialTex row
    (programs per p index; k = 0 is the colour)."""
    rec = np.zeros(20, np.float32)
    t = n.child("type").s
    rec[0] = MAT_TYPES[t]
    st = n.find("shadow_terminator_term")
    rec[1] = 1.0 if st is None or st.s == "true" else 0.0
    p = rec[2:18]
    row = np.zeros((), MATTEX_DT)
    row["prog"][:] = -1
    row["normal"] = -1
    textured = False

    def comp(node):
        return T.compile(node, vvec3, vfloat, lambda m: parse_transform2d(m, vfloat, vangle_rad))

    def spec(k, node):
        nonlocal textured
        c, prog = comp(node)
        if prog is None:
            p[k:k + 3] = c
        else:
            row["prog"][k] = prog
            textured = True

    def scal(k, node, default):
        nonlocal textured
        if node is None:
            p[k] = default
            return
        c, prog = comp(node)
        if prog is None:
            p[k] = c[0]
        else:
            row["prog"][k] = prog
            textured = True

    if t in ("diffuse", "metal", "disney", "glass", "mirror") and n.find("normal") is not None:
        c, prog = comp(n.child("normal"))
        row["normal"] = T.constant_program(c) if prog is None else prog
        textured = True
    if t in ("diffuse", "mirror"):
        spec(0, n.child("color"))
    elif t == "glass":
        spec(0, n.child("color"))
        scal(3, n.child("ior"), 1.5)
    elif t == "metal":
        spec(0, n.child("color"))
        scal(3, n.child("roughness"), 0)
        scal(4, n.find("anisotropic"), 0)
    elif t == "disney":
        spec(0, n.child("color"))
        scal(3, n.child("metallic"), 0)
        scal(4, n.child("roughness"), 0)
        scal(5, n.find("specular"), 1)
        scal(6, n.find("specular_tint"), 0)
        scal(7, n.find("anisotropic"), 0)
        scal(8, n.find("sheen"), 0)
        scal(9, n.find("sheen_tint"), 0)
        scal(10, n.find("clearcoat"), 0)
        scal(11, n.find("clearcoat_gloss"), 1)
        scal(12, n.find("transmission"), 0)
        tr = n.find("transmission_roughness")
        scal(13, tr if tr is not None else n.child("roughness"), 0)
        scal(14, n.find("ior"), 1.5)
    return rec, (row if textured else None)


def _grid(n: Node, sdir: str, rgb: bool = False):
    """Texture3D: constant, {"type":"constant","value":..}, {"type":"array","text":f}
    (common/btrc/utils/cuda/array.cpp:313-384) or {"type":"array","binary":f}.
    Returns (constant, None) or (None, grid[d, h, w] or grid[d, h, w, 3] when rgb and the
    array has 3 or 4 channels). The constant is the red channel, or [r, g, b] when rgb.
    "byte" components are single characters read as signed 8-bit normalised values."""
    if n.kind in ("value", "array"):
        v = vvec3(n)
        return (v if rgb else float(v[0])), None
    t = n.child("type").s
    if t == "constant":
        v = vvec3(n.child("value"))
        return (v if rgb else float(v[0])), None
    if t != "array":
        raise ValueError("texture3d type " + t)
    if n.find("binary") is not None:
        fn = n.child("binary").s.replace("$env{scene_directory}", sdir)
        raw = Path(fn).read_bytes()
        assert raw[:4] == b"BTG1"
        w, h, d = np.frombuffer(raw[4:16], np.int32)
        return None, np.frombuffer(raw[16:], np.float32, count=int(w) * int(h) * int(d)).reshape(int(d), int(h), int(w))
    fn = n.child("text").s.replace("$env{scene_directory}", sdir)
    toks = Path(fn).read_text().split()
    comp, ch, w, h, d = toks[0], int(toks[1]), int(toks[2]), int(toks[3]), int(toks[4])
    count = ch * w * h * d
    if comp == "byte":
        chars = "".join(toks[5:]).encode("latin-1")[:count]
        vals = np.frombuffer(chars, np.int8).astype(np.float64) / 127.0
        vals = np.maximum(vals, -1.0)
    else:
        vals = np.array(toks[5:5 + count], np.float64)
    vals = vals.reshape(-1, ch)
    if rgb and ch > 1:
        return None, vals[:, :3].astype(np.float32).reshape(d, h, w, 3)
    return None, vals[:, 0].astype(np.float32).reshape(d, h, w)


def _volume(n: Node, sdir: str):
    """One volume primitive (factory/btrc/factory/scene.cpp:57-79): the 32-float record of
    oracle.cpp's volume() and its sigma_t / albedo grids (or None)."""
    rec = np.zeros(32, np.float32)
    for k, key in enumerate(("o", "x", "y", "z")):
        rec[3 * k:3 * k + 3] = vvec3(n.child(key))
    c, sg = _grid(n.child("sigma_t"), sdir)
    if sg is None:
        rec[12] = rec[13] = c
        rec[14:17] = 1
    else:
        rec[13] = float(sg.max())
        rec[14], rec[15], rec[16] = sg.shape[2], sg.shape[1], sg.shape[0]
        rec[24] = 1
    ca, ag = _grid(n.child("albedo"), sdir, rgb=True)
    if ag is None:
        rec[21:24] = ca
        rec[17:20] = 1
        rec[20] = 3
    else:
        rec[17], rec[18], rec[19] = ag.shape[2], ag.shape[1], ag.shape[0]
        rec[20] = 3 if ag.ndim == 4 else 1
        rec[25] = 1
    return rec, sg, ag


def volume_box(rec: np.ndarray):
    """VolumePrimitive::get_bounding_box (core/btrc/core/volume.cpp:54-68)."""
    o, x, y, z = rec[0:3], rec[3:6], rec[6:9], rec[9:12]
    pts = np.stack([o, (o + x).astype(np.float32), (o + y).astype(np.float32), (o + z).astype(np.float32)])
    return pts.min(0), pts.max(0)


def _medium(n: Node, sdir: str, w2l=None):
    """One medium record (28 floats) + grid; transform media compose their world-to-local."""
    t = n.child("type").s
    if t == "transform":
        if n.find("world_to_local") is not None:
            mat, _inv = parse_transform(n.child("world_to_local"))
        else:
            _m, mat = parse_transform(n.child("local_to_world"))
        mat = mat if w2l is None else mat_mul(mat, w2l)
        return _medium(n.child("medium"), sdir, mat)
    rec = np.zeros(28, np.float32)
    m = w2l if w2l is not None else np.eye(4, dtype=np.float32)
    rec[12:24] = m[:3].reshape(-1)
    pr = n.find("priority")
    prio = float(vfloat(pr)) if pr is not None else 0.0
    rec[1] = prio
    grid = None
    if t == "homogeneous":
        rec[0] = 1
        rec[8] = vfloat(n.child("sigma_t"))
        rec[9:12] = vvec3(n.child("albedo"))
        rec[7] = vfloat(n.child("g")) if n.find("g") is not None else 0.0
    elif t in ("hetergeneous", "heterogeneous"):
        rec[0] = 2
        c, grid = _grid(n.child("sigma_t"), sdir)
        if grid is None:
            grid = np.array([[[c]]], np.float32)
        rec[2], rec[3], rec[4] = grid.shape[2], grid.shape[1], grid.shape[0]
        rec[6] = max(float(grid.max()), 0.001)
        alb = n.child("albedo")
        rec[9:12] = vvec3(alb.child("value")) if alb.kind == "group" else vvec3(alb)
        rec[7] = _grid(n.child("g"), sdir)[0] if n.find("g") is not None else 0.0
    else:
        raise ValueError("medium type " + t)
    return rec, grid, prio


class Scene:
    """Flattened oracle scene; keeps every array alive for the C side."""

    def __init__(self, path: str | os.PathLike):
        root, sdir = parse_scene_json(path)
        self.width = int(root.child("width").s)
        self.height = int(root.child("height").s)
        cam = root.child("camera")
        eye, dst, up = vvec3(cam.child("eye")), vvec3(cam.child("dst")), vvec3(cam.child("up"))
        fov = vangle_deg(cam.child("fov_y"))
        self.camera = _pinhole(eye, dst, up, fov, f32(f32(self.width) / f32(self.height)))
        r = root.child("renderer")

        def rint(k, d):
            return int(r.find(k).s) if r.find(k) is not None else d

        def rflt(k, d):
            return float(vfloat(r.find(k))) if r.find(k) is not None else d

        self.spp = rint("spp", 128)
        self.min_depth, self.max_depth = rint("min_depth", 5), rint("max_depth", 10)
        self.rr_threshold, self.rr_cont_prob = rflt("rr_threshold", 0.1), rflt("rr_cont_prob", 0.5)
        smp = r.find("sampler")
        self.sampler = 1 if smp is not None and (smp.s if smp.kind == "value" else smp.child("type").s) == "halton" else 0
        flt = r.find("filter")
        self.filter, self.filter_radius, self.filter_alpha = 0, 1.3, 1.6
        if flt is not None and flt.child("type").s == "gaussian":
            self.filter = 1
            self.filter_radius = float(vfloat(flt.child("radius"))) if flt.find("radius") is not None else 1.3
            self.filter_alpha = float(vfloat(flt.child("alpha"))) if flt.find("alpha") is not None else 1.6

        scene = root.child("scene")
        geo_ids: dict[int, int] = {}
        mat_ids: dict[int, int] = {}
        geos, mats = [], []
        inst = []
        med_ids: dict[int, int] = {}
        meds = []
        self.tex = TexStore(sdir)
        mat_rows, mat_texrow = [], []
        for e in scene.child("entities").elems:
            gn = e.child("geometry")
            if id(gn) not in geo_ids:
                gtype = gn.child("type").s
                if gtype == "triangle_mesh":
                    fn = gn.child("filename").s.replace("$env{scene_directory}", sdir)
                    unit = gn.find("transform_to_unit_cube")
                    geos.append(load_obj(fn, unit is not None and unit.s == "true"))
                else:
                    sub = gn.find("subdivisions")
                    geos.append(procedural(gtype, int(vfloat(sub)) if sub is not None else 3))
                geo_ids[id(gn)] = len(geos) - 1
            mn = e.child("material")
            if id(mn) not in mat_ids:
                rec, row = _material(mn, self.tex)
                mats.append(rec)
                if row is not None:
                    mat_texrow.append(len(mat_rows))
                    mat_rows.append(row)
                else:
                    mat_texrow.append(-1)
                mat_ids[id(mn)] = len(mats) - 1
            xf = parse_transform(e.child("local_to_world")) if e.find("local_to_world") is not None else \
                (np.eye(4, dtype=np.float32), np.eye(4, dtype=np.float32))
            light = e.find("light")
            inten = vvec3(light.child("intensity")) if light is not None else None
            media = []
            for key in ("inner_medium", "outer_medium"):
                mnode = e.find(key)
                if mnode is None:
                    media.append(-1)
                    continue
                if id(mnode) not in med_ids:
                    meds.append(_medium(mnode, sdir))
                    med_ids[id(mnode)] = len(meds) - 1
                media.append(med_ids[id(mnode)])
            inst.append((geo_ids[id(gn)], mat_ids[id(mn)], xf, inten, media))

        self.geos = geos
        counts = np.array([len(g[2]) for g in geos], np.uint64)
        self.geo_offset = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint64)
        self.geo_count = counts
        self.geo_area_total = np.array([float(np.sum(g[2], dtype=np.float64)) for g in geos], np.float32)
        # a scene without entities has no geometry: empty tables of the same layouts
        self.shade = np.ascontiguousarray(np.concatenate([g[1] for g in geos], axis=1) if geos
                                          else np.zeros((6, 0, 4)), np.float32)
        self.tri_area = np.ascontiguousarray(np.concatenate([g[2] for g in geos]) if geos else np.zeros(0), np.float32)
        self.local_pos = np.ascontiguousarray(np.concatenate([g[0].reshape(-1, 9) for g in geos]) if geos
                                              else np.zeros((0, 9)), np.float32)
        self.mat = np.ascontiguousarray(np.stack(mats) if mats else np.zeros((1, 20)), np.float32)

        tris, ids = [], []
        l2w, w2l, igeo, imat, ilight = [], [], [], [], []
        linst, lgeo, lscale, lint = [], [], [], []
        # medium table (core/btrc/core/scene.cpp:136-161): priority descending, creation
        # order on ties, the volume-primitive medium (vacuum) last
        order = sorted(range(len(meds)), key=lambda k: -meds[k][2])
        remap = {k: i for i, k in enumerate(order)}
        recs, offs, grids, off = [], [], [], 0
        for k in order:
            rec, grid, _ = meds[k]
            recs.append(rec)
            offs.append(off)
            if grid is not None:
                grids.append(grid.reshape(-1))
                off += grid.size
        # volume primitives: their grids follow the media grids in the same pool
        vol_recs, vol_offs = [], []
        vnode = scene.find("volumes")
        for vn in (vnode.elems if vnode is not None else []):
            rec, sg, ag = _volume(vn, sdir)
            so = ao = 0
            if sg is not None:
                so = off
                grids.append(sg.reshape(-1))
                off += sg.size
            if ag is not None:
                ao = off
                grids.append(ag.reshape(-1))
                off += ag.size
            vol_recs.append(rec)
            vol_offs += [so, ao]
        self.vol = np.ascontiguousarray(np.stack(vol_recs) if vol_recs else np.zeros((1, 32)), np.float32)
        self.vol_off = np.array(vol_offs if vol_offs else [0, 0], np.uint64)
        self.nvol = len(vol_recs)
        vac = np.zeros(28, np.float32)
        vac[0] = 3 if self.nvol else 0
        vac[1] = -1e30
        recs.append(vac)
        offs.append(off)
        self.vacuum = len(recs) - 1
        self.med = np.ascontiguousarray(np.stack(recs), np.float32)
        self.med_grid_offset = np.array(offs, np.uint64)
        self.grids = np.ascontiguousarray(np.concatenate(grids) if grids else np.zeros(1, np.float32), np.float32)
        inner, outer = [], []
        for *_, media in inst:
            inner.append(self.vacuum if media[0] < 0 else remap[media[0]])
            outer.append(self.vacuum if media[1] < 0 else remap[media[1]])
        for i, (g, m, (mat, inv), inten, _media) in enumerate(inst):
            pos = geos[g][0].reshape(-1, 3)
            w = apply_point(mat, pos).reshape(-1, 9)
            tris.append(w)
            ids.append(np.stack([np.full(len(w), i, np.uint32), np.arange(len(w), dtype=np.uint32)], 1))
            l2w.append(mat[:3].reshape(-1))
            w2l.append(inv[:3].reshape(-1))
            igeo.append(g)
            imat.append(m)
            if inten is not None:
                ilight.append(len(linst))
                linst.append(i)
                lgeo.append(g)
                p1 = apply_point(mat, np.array([[1, 0, 0]], np.float32))[0]
                p0 = apply_point(mat, np.array([[0, 0, 0]], np.float32))[0]
                dd = (p1 - p0).astype(np.float32)
                lscale.append(f32(np.sqrt(f32(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]))))
                lint.append(inten)
            else:
                ilight.append(-1)
        self.tris = np.ascontiguousarray(np.concatenate(tris) if tris else np.zeros((0, 9)), np.float32)
        self.ids = np.ascontiguousarray(np.concatenate(ids) if ids else np.zeros((0, 2)), np.uint32)
        self.inst_l2w = np.ascontiguousarray(np.stack(l2w) if l2w else np.zeros((1, 12)), np.float32)
        self.inst_w2l = np.ascontiguousarray(np.stack(w2l) if w2l else np.zeros((1, 12)), np.float32)
        self.inst_geo = np.array(igeo, np.int32)
        self.inst_mat = np.array(imat, np.int32)
        self.inst_light = np.array(ilight, np.int32)
        self.inst_inner = np.array(inner, np.int32)
        self.inst_outer = np.array(outer, np.int32)
        # world bounds (core/btrc/core/scene.cpp:224-236): transformed geometry boxes
        lo, hi = np.full(3, np.inf, np.float32), np.full(3, -np.inf, np.float32)
        for i, (g, m, (mat, inv), inten, _media) in enumerate(inst):
            pos = geos[g][0].reshape(-1, 3)
            if not len(pos):
                continue
            bl, bh = pos.min(0), pos.max(0)
            corners = np.array([[bh[0] if c & 1 else bl[0], bh[1] if c & 2 else bl[1], bh[2] if c & 4 else bl[2]]
                                for c in range(8)], np.float32)
            w = apply_point(mat, corners)
            lo, hi = np.minimum(lo, w.min(0)), np.maximum(hi, w.max(0))
        # volume boxes join the world bounds (core/btrc/core/scene.cpp:233-237)
        for k in range(self.nvol):
            bl, bh = volume_box(self.vol[k])
            lo, hi = np.minimum(lo, bl), np.maximum(hi, bh)
        if not np.all(lo <= hi):
            lo, hi = np.zeros(3, np.float32), np.zeros(3, np.float32)
        ext = (hi - lo).astype(np.float32)
        self.world_diagonal = float(np.sqrt(np.float32((ext * ext).sum(dtype=np.float32))))
        self.light_inst = np.array(linst, np.int32)
        self.light_geo = np.array(lgeo, np.int32)
        self.light_scale = np.array(lscale, np.float32)
        self.light_intensity = np.ascontiguousarray(np.array(lint, np.float32).reshape(-1, 3))
        self.env = None
        self.env_ibl = None
        en = scene.find("envir_light")
        if en is not None:
            et = en.child("type").s
            if et == "gradient_sky":
                upv = vvec3(en.child("up"))
                self.env = (vvec3(en.child("lower")), vvec3(en.child("upper")), _nrm(upv[None])[0])
            elif et == "ibl":
                # IBLCreator (builtin/btrc/builtin/light/ibl.cpp:80-91); oracle.cpp builds
                # the frame from "up" and the tile table itself
                c, prog = self.tex.compile(en.child("tex"), vvec3, vfloat,
                                           lambda m: parse_transform2d(m, vfloat, vangle_rad))
                prog = self.tex.constant_program(c) if prog is None else prog
                upv = vvec3(en.child("up")) if en.find("up") is not None else np.array([0, 0, 1], np.float32)
                lw = int(vfloat(en.child("lut_width"))) if en.find("lut_width") is not None else 400
                lh = int(vfloat(en.child("lut_height"))) if en.find("lut_height") is not None else 200
                self.env_ibl = (prog, upv, lw, lh)
            else:
                raise ValueError("environment light " + et)
        self.mat_tex = np.ascontiguousarray(np.stack(mat_rows) if mat_rows else np.zeros(1, MATTEX_DT))
        self.mat_texrow = np.array(mat_texrow, np.int32)
        self.tex_img, self.tex_texels, self.tex_instr = self.tex.arrays()
        self._prepared = None

    def struct(self) -> OracleScene:
        s = OracleScene()
        s.tris, s.ids, s.ntri = _p(self.tris), _p(self.ids), len(self.tris)
        s.ninst = len(self.inst_geo)
        s.inst_l2w, s.inst_w2l = _p(self.inst_l2w), _p(self.inst_w2l)
        s.inst_geo, s.inst_mat, s.inst_light = _p(self.inst_geo), _p(self.inst_mat), _p(self.inst_light)
        s.inst_inner, s.inst_outer = _p(self.inst_inner), _p(self.inst_outer)
        s.ngeo = len(self.geos)
        s.geo_offset, s.geo_count, s.geo_area_total = _p(self.geo_offset), _p(self.geo_count), _p(self.geo_area_total)
        s.shade, s.total_geo_tris = _p(self.shade), self.shade.shape[1]
        s.tri_area, s.local_pos = _p(self.tri_area), _p(self.local_pos)
        s.nmat, s.mat = len(self.mat), _p(self.mat)
        s.nlight = len(self.light_inst)
        if s.nlight:
            s.light_inst, s.light_geo = _p(self.light_inst), _p(self.light_geo)
            s.light_scale, s.light_intensity = _p(self.light_scale), _p(self.light_intensity)
        if self.env is not None:
            s.env_type = 1
            s.env_lower[:], s.env_upper[:], s.env_up[:] = [list(map(float, v)) for v in self.env]
        if self.env_ibl is not None:
            s.env_type = 2
            s.env_prog, up, s.env_lut_w, s.env_lut_h = self.env_ibl
            s.env_up[:] = list(map(float, up))
        s.ntex_img = len(self.tex.images)
        s.tex_img, s.tex_texels, s.tex_instr = _p(self.tex_img), _p(self.tex_texels), _p(self.tex_instr)
        s.mat_tex, s.mat_texrow = _p(self.mat_tex), _p(self.mat_texrow)
        s.vacuum_medium = self.vacuum
        s.world_diagonal = self.world_diagonal
        s.nmed, s.med, s.med_grid_offset, s.grids = len(self.med), _p(self.med), _p(self.med_grid_offset), _p(self.grids)
        eye, lbc, fx, fy = self.camera
        s.eye[:], s.lbc[:], s.film_x[:], s.film_y[:] = (list(map(float, v)) for v in (eye, lbc, fx, fy))
        s.width, s.height, s.spp = self.width, self.height, self.spp
        s.min_depth, s.max_depth = self.min_depth, self.max_depth
        s.rr_threshold, s.rr_cont_prob = self.rr_threshold, self.rr_cont_prob
        s.sampler, s.filter = self.sampler, self.filter
        s.filter_radius, s.filter_alpha = self.filter_radius, self.filter_alpha
        s.nvol, s.vol, s.vol_off = self.nvol, _p(self.vol), _p(self.vol_off)
        return s

    def medium_tr(self, medium_id: int, seg: np.ndarray, seeds: np.ndarray) -> np.ndarray:
        """Ratio-tracking transmittance of segments (n, 6) through one medium, one PCG
        stream per segment seeded (seeds[i], PCG_STREAM)."""
        seg = np.ascontiguousarray(seg, np.float32)
        seeds = np.ascontiguousarray(seeds, np.uint64)
        out = np.zeros(len(seg), np.float32)
        st = self.struct()
        lib().oracle_medium_tr_batch(st, medium_id, _p(seg), _p(seeds), len(seg), _p(out))
        return out

    def prepare(self):
        if self._prepared is None:
            self._struct = self.struct()
            self._prepared = lib().oracle_prepare(self._struct)
        return self._prepared

    def render(self, spp: int | None = None, sample_begin: int = 0, pixel_begin: int = 0, pixel_end: int | None = None,
               threads: int = 0) -> np.ndarray:
        """Film (H, W, 4) float64: radiance sums and weights for the requested range."""
        h = self.prepare()
        spp = self.spp if spp is None else spp
        film = np.zeros((self.height, self.width, 4), np.float64)
        pe = self.width * self.height if pixel_end is None else pixel_end
        lib().oracle_render(h, pixel_begin, pe, sample_begin, sample_begin + spp, _p(film), threads)
        return film

    def render_aov(self, spp: int | None = None, sample_begin: int = 0, threads: int = 0):
        """Film (H, W, 4) and first-hit g-buffer sums (H, W, 6): albedo.rgb, normal.xyz."""
        h = self.prepare()
        spp = self.spp if spp is None else spp
        film = np.zeros((self.height, self.width, 4), np.float64)
        aov = np.zeros((self.height, self.width, 6), np.float64)
        lib().oracle_render_aov(h, 0, self.width * self.height, sample_begin, sample_begin + spp, _p(film), _p(aov),
                                threads)
        return film, aov

    def __del__(self):
        try:
            if self._prepared is not None:
                lib().oracle_release(self._prepared)
        except Exception:
            pass


def _pinhole(eye, dst, up, fov_deg, w_over_h):
    fwd = _nrm((dst - eye)[None])[0]
    ex = _nrm(_cross(fwd, up)[None])[0]
    ey = _nrm(_cross(fwd, ex)[None])[0]
    y_len = f32(2) * f32(math.tan(float(f32(f32(0.5) * fov_deg * f32(math.pi) / f32(180)))))
    x_len = f32(w_over_h * y_len)
    lbc = (eye + fwd - f32(0.5) * (x_len * ex + y_len * ey)).astype(np.float32)
    return eye, lbc, (x_len * ex).astype(np.float32), (y_len * ey).astype(np.float32)


def resolve(film: np.ndarray) -> np.ndarray:
    w = film[..., 3:4]
    return np.where(w > 0, film[..., :3] / np.maximum(w, 1e-300), 0.0)


def resolve_aov(film: np.ndarray, aov: np.ndarray):
    """The preview resolve of the g-buffer (wavefront/preview.cpp:27-78): albedo = sum /
    weight; normal = sum / weight renormalised, zero when shorter than 1e-3."""
    w = film[..., 3:4]
    alb = np.where(w > 0, aov[..., 0:3] / np.maximum(w, 1e-300), 0.0)
    n = np.where(w > 0, aov[..., 3:6] / np.maximum(w, 1e-300), 0.0)
    ln = np.linalg.norm(n, axis=-1, keepdims=True)
    n = np.where(ln > 1e-3, n / np.maximum(ln, 1e-300), 0.0)
    return alb, n
