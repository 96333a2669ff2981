"""Seeded synthetic scenes in Btrc's scene-JSON schema (OBJ geometry + JSON).

The reference ships no scenes, so the benchmark and parity workloads are generated:

  cornell  : closed box of unit cross-section (12 triangles in three entities, normals
             facing inwards, deepened towards the camera), two level-3
             icospheres (1280 triangles, radius 0.3) at seeded positions, a 0.25 x 0.25
             quad light of radiance 15 under the ceiling, Lambertian albedos U[0.2, 0.8]^3,
             pinhole 40 degrees, 256x256, 16 spp, max depth 8, Russian roulette from depth 3,
             Halton sampler, Gaussian filter of radius 1.5.
  terrain  : 1024x1024-vertex fBm heightfield (8 octaves, amplitude 0.2, lacunarity 2,
             Perlin gradient noise), 200 instances of one level-4 icosphere, Disney
             materials (base colour U[0,1]^3, roughness U[0.05,1], metallic Bernoulli(0.3),
             specular 0.5, clearcoat U[0,1]), gradient sky + 8 quad lights, 1920x1080,
             64 spp, depth 16.
  volume   : the cornell box with a 256^3 fBm density grid (sigma_t max 20, albedo 0.9,
             g 0.6) inside an invisible cube, plus a noise-displaced level-7 icosphere with
             a GGX conductor of roughness 0.2; 1024x1024, 64 spp, depth 32.

Every random choice draws from numpy's PCG64 seeded with the scene seed.
"""
from __future__ import annotations

import json
import struct
import os
from pathlib import Path

import numpy as np

CACHE_ENV = "BTRC_SCENE_CACHE"


def cache_dir() -> Path:
    d = Path(os.environ.get(CACHE_ENV, "/tmp/btrc_gb300_scenes"))
    d.mkdir(parents=True, exist_ok=True)
    return d


# ------------------------------------------------------------------ geometry helpers

def icosphere(level: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: (V, 3) float64 vertices and (F, 3) int faces, 20 * 4^level faces."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(level):
        cache: dict[tuple[int, int], int] = {}

        def mid(a: int, b: int) -> int:
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts), np.array(faces, np.int64)


def write_obj(path: Path, verts: np.ndarray, faces: np.ndarray, normals: np.ndarray | None = None,
              uvs: np.ndarray | None = None) -> None:
    """OBJ with 1-based indices; with normals, faces are written as a//a, with normals and
    per-vertex texture coordinates as a/a/a."""
    verts = np.asarray(verts, np.float64)
    faces = np.asarray(faces, np.int64) + 1
    parts = [("v %.7g %.7g %.7g\n" * len(verts)) % tuple(verts.ravel())]
    if uvs is not None:
        assert normals is not None
        normals = np.asarray(normals, np.float64)
        uvs = np.asarray(uvs, np.float64)
        parts.append(("vt %.7g %.7g\n" * len(uvs)) % tuple(uvs.ravel()))
        parts.append(("vn %.6g %.6g %.6g\n" * len(normals)) % tuple(normals.ravel()))
        ff = np.repeat(faces, 3, axis=1)
        parts.append(("f %d/%d/%d %d/%d/%d %d/%d/%d\n" * len(faces)) % tuple(ff.ravel()))
    elif normals is not None:
        normals = np.asarray(normals, np.float64)
        parts.append(("vn %.6g %.6g %.6g\n" * len(normals)) % tuple(normals.ravel()))
        ff = np.repeat(faces, 2, axis=1)
        parts.append(("f %d//%d %d//%d %d//%d\n" * len(faces)) % tuple(ff.ravel()))
    else:
        parts.append(("f %d %d %d\n" * len(faces)) % tuple(faces.ravel()))
    tmp = path.with_suffix(path.suffix + ".tmp")
    with open(tmp, "w") as fobj:
        for p in parts:
            fobj.write(p)
    os.replace(tmp, path)


def write_png(path: Path, img: np.ndarray, depth: int = 8, palette: np.ndarray | None = None,
              alpha: np.ndarray | None = None) -> None:
    """PNG writer for test textures: 8/16-bit grey (H, W), RGB (H, W, 3) or RGBA (H, W, 4),
    low-depth grey (depth 1/2/4), or palette indices (H, W) with `palette` (N, 3) and an
    optional tRNS `alpha`. Rows cycle through the five filter types; zlib level 6."""
    import zlib
    img = np.asarray(img)
    h, w = img.shape[:2]
    if palette is not None:
        ctype, samples = 3, 1
    else:
        samples = 1 if img.ndim == 2 else img.shape[2]
        ctype = {1: 0, 3: 2, 4: 6}[samples]
    if depth < 8:
        bits = np.unpackbits(img.astype(np.uint8)[..., None], axis=-1)[..., 8 - depth:]
        rows = np.packbits(bits.reshape(h, -1), axis=1)
    elif depth == 16:
        rows = img.astype(">u2").reshape(h, -1).view(np.uint8).reshape(h, -1)
    else:
        rows = img.astype(np.uint8).reshape(h, -1)
    bpp = max(1, samples * depth // 8)
    out = bytearray()
    prev = np.zeros(rows.shape[1], np.int32)
    for y in range(h):
        cur = rows[y].astype(np.int32)
        ft = y % 5
        left = np.concatenate([np.zeros(bpp, np.int32), cur[:-bpp]])
        ul = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        if ft == 0:
            f = cur
        elif ft == 1:
            f = cur - left
        elif ft == 2:
            f = cur - prev
        elif ft == 3:
            f = cur - (left + prev) // 2
        else:
            pa, pb, pc = np.abs(prev - ul), np.abs(left - ul), np.abs(left + prev - 2 * ul)
            pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, ul))
            f = cur - pred
        out.append(ft)
        out += (f & 255).astype(np.uint8).tobytes()
        prev = cur

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xffffffff)
    data = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
    if palette is not None:
        data += chunk(b"PLTE", np.asarray(palette, np.uint8).tobytes())
        if alpha is not None:
            data += chunk(b"tRNS", np.asarray(alpha, np.uint8).tobytes())
    data += chunk(b"IDAT", zlib.compress(bytes(out), 6)) + chunk(b"IEND", b"")
    Path(path).write_bytes(data)


def write_hdr(path: Path, rgb: np.ndarray) -> None:
    """Radiance RGBE file, adaptive run-length encoded scanlines."""
    rgb = np.maximum(np.asarray(rgb, np.float64), 0)
    h, w = rgb.shape[:2]
    m = rgb.max(-1)
    e = np.where(m > 1e-32, np.floor(np.log2(np.maximum(m, 1e-32))) + 1, 0)
    scale = np.where(m > 1e-32, 256.0 / np.exp2(e), 0)
    rgbe = np.zeros((h, w, 4), np.uint8)
    rgbe[..., :3] = np.clip(rgb * scale[..., None], 0, 255).astype(np.uint8)
    rgbe[..., 3] = np.where(m > 1e-32, e + 128, 0).astype(np.uint8)
    out = bytearray(f"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y {h} +X {w}\n".encode())
    for y in range(h):
        out += bytes([2, 2, w >> 8, w & 255])
        for c in range(4):
            row = rgbe[y, :, c]
            x = 0
            while x < w:
                run = 1
                while x + run < w and run < 127 and row[x + run] == row[x]:
                    run += 1
                if run >= 4:
                    out += bytes([128 + run, row[x]])
                    x += run
                else:
                    n = 1
                    while x + n < w and n < 128 and not (x + n + 2 < w and row[x + n] == row[x + n + 1] == row[x + n + 2]):
                        n += 1
                    out += bytes([n]) + row[x:x + n].tobytes()
                    x += n
    Path(path).write_bytes(bytes(out))


def quad(size: float = 1.0) -> tuple[np.ndarray, np.ndarray]:
    """Square in the xz plane, centred at the origin, normal +y."""
    h = size / 2
    v = np.array([[-h, 0, -h], [h, 0, -h], [h, 0, h], [-h, 0, h]], np.float64)
    f = np.array([[0, 2, 1], [0, 3, 2]], np.int64)
    return v, f


def flip(faces: np.ndarray) -> np.ndarray:
    return faces[:, [0, 2, 1]]


def box_inward(lo, hi) -> tuple[np.ndarray, np.ndarray]:
    """Closed axis-aligned box [lo, hi] of 12 triangles with normals facing inwards.
    Faces in order: x-, x+, y-, y+, z-, z+ (two triangles each)."""
    v = np.array([[x, y, z] for x in (lo[0], hi[0]) for y in (lo[1], hi[1]) for z in (lo[2], hi[2])], np.float64)
    # vertex index = 4*ix + 2*iy + iz
    quads = [
        (0, 1, 3, 2),  # x = -h
        (4, 6, 7, 5),  # x = +h
        (0, 4, 5, 1),  # y = -h
        (2, 3, 7, 6),  # y = +h
        (0, 2, 6, 4),  # z = -h
        (1, 5, 7, 3),  # z = +h
    ]
    f = []
    for a, b, c, d in quads:
        f += [(a, b, c), (a, c, d)]
    f = np.array(f, np.int64)
    # orient every face towards the centre
    tri = v[f]
    n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    c = tri.mean(axis=1) - 0.5 * (np.asarray(lo) + np.asarray(hi))
    wrong = np.einsum("ij,ij->i", n, -c) < 0
    f[wrong] = f[wrong][:, [0, 2, 1]]
    return v, f


# ------------------------------------------------------------------ noise

class Perlin:
    """Improved gradient noise (Perlin 2002) with a seeded permutation table."""

    def __init__(self, rng: np.random.Generator):
        p = rng.permutation(256)
        self.p = np.concatenate([p, p]).astype(np.int64)

    @staticmethod
    def _fade(t):
        return t * t * t * (t * (t * 6 - 15) + 10)

    @staticmethod
    def _grad(h, x, y, z):
        h = h & 15
        u = np.where(h < 8, x, y)
        v = np.where(h < 4, y, np.where((h == 12) | (h == 14), x, z))
        return np.where(h & 1, -u, u) + np.where(h & 2, -v, v)

    def noise3(self, x, y, z):
        X = np.floor(x).astype(np.int64) & 255
        Y = np.floor(y).astype(np.int64) & 255
        Z = np.floor(z).astype(np.int64) & 255
        x = x - np.floor(x)
        y = y - np.floor(y)
        z = z - np.floor(z)
        u, v, w = self._fade(x), self._fade(y), self._fade(z)
        p = self.p
        A = p[X] + Y
        AA = p[A] + Z
        AB = p[A + 1] + Z
        B = p[X + 1] + Y
        BA = p[B] + Z
        BB = p[B + 1] + Z
        g = self._grad
        lerp = lambda t, a, b: a + t * (b - a)
        return lerp(w,
                    lerp(v, lerp(u, g(p[AA], x, y, z), g(p[BA], x - 1, y, z)),
                         lerp(u, g(p[AB], x, y - 1, z), g(p[BB], x - 1, y - 1, z))),
                    lerp(v, lerp(u, g(p[AA + 1], x, y, z - 1), g(p[BA + 1], x - 1, y, z - 1)),
                         lerp(u, g(p[AB + 1], x, y - 1, z - 1), g(p[BB + 1], x - 1, y - 1, z - 1))))

    def fbm3(self, x, y, z, octaves=8, lacunarity=2.0, gain=0.5):
        total = np.zeros_like(np.asarray(x, np.float64))
        amp, freq = 1.0, 1.0
        for _ in range(octaves):
            total += amp * self.noise3(x * freq, y * freq, z * freq)
            amp *= gain
            freq *= lacunarity
        return total


# ------------------------------------------------------------------ scene JSON helpers

def _entity(geometry, material, transform=None, light=None, inner=None, outer=None) -> dict:
    e = {"geometry": geometry, "material": material}
    if transform is not None:
        e["local_to_world"] = transform
    if inner is not None:
        e["inner_medium"] = inner
    if outer is not None:
        e["outer_medium"] = outer
    if light is not None:
        e["light"] = light
    return e


def _diffuse(rgb) -> dict:
    return {"type": "diffuse", "color": [float(c) for c in rgb]}


def _write_scene(path: Path, scene: dict) -> Path:
    tmp = path.with_suffix(".json.tmp")
    tmp.write_text(json.dumps(scene, indent=1))
    os.replace(tmp, path)
    return path


# ------------------------------------------------------------------ configurations

SPHERE_VARIANTS = {
    # materials of the two spheres; None = diffuse with a seeded albedo
    "diffuse": (None, None),
    # a smooth-shaded glass sphere (ior 1.5, builtin/btrc/builtin/material/glass.cpp) and a
    # tinted mirror (mirror.cpp): delta reflection + refraction, no light sampling on either
    "glass": ({"type": "glass", "color": [0.95, 0.97, 1.0], "ior": 1.5},
              {"type": "mirror", "color": [0.9, 0.8, 0.6]}),
    # diffuse spheres inside three overlapping volume primitives (volumes[])
    "fog": (None, None),
}


def _fog_volumes(out: Path, rng: np.random.Generator) -> list[dict]:
    """Three overlapping volume primitives (core/btrc/core/volume.h): an axis-aligned box of
    constant density, a sheared box with an 8^3 density grid and a coloured box whose albedo
    is a 4^3 RGB grid (text array files, common/btrc/utils/cuda/array.cpp:313-384)."""
    sig = rng.uniform(0.0, 4.0, (8, 8, 8)).astype(np.float32)
    write_grid_text(out / "fog_sigma.txt", sig)
    alb = rng.uniform(0.2, 0.95, (4, 4, 4, 3)).astype(np.float32)
    lines = ["float 3 4 4 4"] + [" ".join(f"{v:.6f}" for v in t) for t in alb.reshape(-1, 3)]
    (out / "fog_albedo.txt").write_text("\n".join(lines) + "\n")
    return [
        {"o": [-0.45, -0.45, 0.25], "x": [0.55, 0.0, 0.0], "y": [0.0, 0.5, 0.0], "z": [0.0, 0.0, 0.6],
         "sigma_t": 2.0, "albedo": 0.8},
        {"o": [-0.15, -0.35, 0.4], "x": [0.45, 0.12, 0.0], "y": [-0.1, 0.45, 0.05], "z": [0.0, 0.0, 0.5],
         "sigma_t": {"type": "array", "text": "$env{scene_directory}/fog_sigma.txt"},
         "albedo": [0.9, 0.5, 0.3]},
        {"o": [-0.3, 0.0, 0.3], "x": [0.6, 0.0, 0.0], "y": [0.0, 0.35, 0.0], "z": [0.0, 0.0, 0.4],
         "sigma_t": 1.0,
         "albedo": {"type": "array", "text": "$env{scene_directory}/fog_albedo.txt"}},
    ]


def cornell(seed: int = 1000, width: int = 256, height: int = 256, spp: int = 16, sampler: str = "halton",
            out_dir: Path | None = None, force: bool = False, variant: str = "diffuse",
            state_count: int = 32 * 1024 * 1024) -> Path:
    """Config 0: closed unit box, two icospheres, one quad light (see module docstring).
    `variant` picks the spheres' materials from SPHERE_VARIANTS."""
    mats = SPHERE_VARIANTS[variant]
    out = Path(out_dir or cache_dir() / f"cornell-{seed}")
    out.mkdir(parents=True, exist_ok=True)
    tag = "" if variant == "diffuse" else f"-{variant}"
    name = f"scene-{width}x{height}-{spp}-{sampler}{tag}-q{state_count}.json"
    if (out / name).exists() and not force:
        return out / name
    rng = np.random.default_rng(seed)
    half = 0.5
    # unit cross-section, deepened towards the camera so that a 40 degree view from inside
    # sees the side walls; left wall, right wall and the rest are separate entities
    bv, bf = box_inward((-half, -half, -half), (half, half, 1.4))
    write_obj(out / "box_left.obj", bv, bf[0:2])
    write_obj(out / "box_right.obj", bv, bf[2:4])
    write_obj(out / "box_rest.obj", bv, bf[4:12])
    sv, sf = icosphere(3)
    write_obj(out / "sphere3.obj", sv, sf, normals=sv)
    qv, qf = quad(0.25)
    write_obj(out / "light.obj", qv, flip(qf))  # normal -y: facing down into the box
    eye = np.array([0.0, 0.0, 1.3])
    radius = 0.3
    centers = []
    while len(centers) < 2:
        c = rng.uniform(-half + radius, half - radius, 3)
        if np.linalg.norm(c - eye) > radius + 0.08:
            centers.append(c)
    albedos = rng.uniform(0.2, 0.8, (6, 3))
    ents = [_entity({"type": "triangle_mesh", "filename": "${" + part + "}"}, _diffuse(albedos[k]))
            for k, part in enumerate(("box_left", "box_right", "box_rest"))]
    for k, c in enumerate(centers):
        ents.append(_entity({"type": "triangle_mesh", "filename": "${sphere}"},
                            mats[k] if mats[k] is not None else _diffuse(albedos[3 + k]),
                            [{"scale": [radius] * 3}, {"translate": [float(x) for x in c]}]))
    ents.append(_entity({"type": "triangle_mesh", "filename": "${light}"}, _diffuse(albedos[5]),
                        [{"translate": [0.0, half - 0.005, 0.0]}],
                        light={"type": "mesh_light", "intensity": [15.0, 15.0, 15.0]}))
    scene = {
        "width": width, "height": height,
        "camera": {"type": "pinhole", "eye": eye.tolist(), "dst": [0.0, 0.0, -half], "up": [0.0, 1.0, 0.0],
                   "fov_y": {"deg": 40.0}},
        "renderer": {"type": "wfpt", "spp": spp, "min_depth": 3, "max_depth": 8, "rr_threshold": 0.1,
                     "rr_cont_prob": 0.5, "state_count": state_count, "sampler": sampler,
                     "filter": {"type": "gaussian", "radius": 1.5, "alpha": 1.6}},
        "scene": {"entities": ents},
    }
    if variant == "fog":
        scene["scene"]["volumes"] = _fog_volumes(out, rng)
    text = json.dumps(scene, indent=1)
    for key, fn in (("${box_left}", "box_left.obj"), ("${box_right}", "box_right.obj"),
                    ("${box_rest}", "box_rest.obj"), ("${sphere}", "sphere3.obj"), ("${light}", "light.obj")):
        text = text.replace(key, "$env{scene_directory}/" + fn)
    (out / name).write_text(text)
    return out / name


def terrain(seed: int = 1001, width: int = 1920, height: int = 1080, spp: int = 64, grid: int = 1024,
            instances: int = 200, out_dir: Path | None = None, force: bool = False,
            state_count: int = 32 * 1024 * 1024) -> Path:
    """Config 1: fBm terrain + instanced icospheres + Disney + sky + 8 quad lights."""
    out = Path(out_dir or cache_dir() / f"terrain-{seed}-{grid}-{instances}")
    out.mkdir(parents=True, exist_ok=True)
    name = f"scene-{width}x{height}-{spp}-q{state_count}.json"
    if (out / name).exists() and not force:
        return out / name
    rng = np.random.default_rng(seed)
    perlin = Perlin(rng)
    # heightfield over [-1, 1]^2 in xz
    xs = np.linspace(-1.0, 1.0, grid)
    X, Z = np.meshgrid(xs, xs, indexing="xy")
    H = 0.2 * perlin.fbm3(X * 2.0 + 0.5, Z * 2.0 + 0.5, np.full_like(X, 0.37), octaves=8, lacunarity=2.0)
    V = np.stack([X, H, Z], axis=-1).reshape(-1, 3)
    # smooth vertex normals from central differences
    dhdx = np.gradient(H, xs, axis=1)
    dhdz = np.gradient(H, xs, axis=0)
    N = np.stack([-dhdx, np.ones_like(H), -dhdz], axis=-1)
    N /= np.linalg.norm(N, axis=-1, keepdims=True)
    idx = np.arange(grid * grid).reshape(grid, grid)
    a, b, c, d = idx[:-1, :-1], idx[:-1, 1:], idx[1:, :-1], idx[1:, 1:]
    F = np.concatenate([np.stack([a, c, b], -1).reshape(-1, 3), np.stack([b, c, d], -1).reshape(-1, 3)])
    write_obj(out / "terrain.obj", V, F, normals=N.reshape(-1, 3))
    sv, sf = icosphere(4)
    write_obj(out / "sphere4.obj", sv, sf, normals=sv)
    qv, qf = quad(1.0)
    write_obj(out / "quad.obj", qv, flip(qf))

    def height_at(x, z):
        return float(0.2 * perlin.fbm3(np.array([x * 2.0 + 0.5]), np.array([z * 2.0 + 0.5]),
                                       np.array([0.37]), octaves=8)[0])

    def disney():
        return {"type": "disney", "color": [float(v) for v in rng.uniform(0, 1, 3)],
                "roughness": float(rng.uniform(0.05, 1.0)),
                "metallic": float(rng.random() < 0.3), "specular": 0.5,
                "clearcoat": float(rng.uniform(0, 1))}

    ents = [_entity({"type": "triangle_mesh", "filename": "$env{scene_directory}/terrain.obj"}, disney())]
    sphere_node = {"type": "triangle_mesh", "filename": "$env{scene_directory}/sphere4.obj"}
    for k in range(instances):
        x, z = rng.uniform(-0.9, 0.9, 2)
        r = float(rng.uniform(0.02, 0.06))
        y = height_at(x, z) + r * float(rng.uniform(0.3, 1.0))
        geo = sphere_node if k == 0 else "$reference{$root/scene/entities/1/geometry}"
        ents.append(_entity(geo, disney(), [{"scale": [r, r, r]}, {"translate": [float(x), y, float(z)]}]))
    for k in range(8):
        x, z = rng.uniform(-0.8, 0.8, 2)
        s = float(rng.uniform(0.05, 0.15))
        y = height_at(x, z) + float(rng.uniform(0.15, 0.4))
        inten = [float(v) for v in rng.uniform(2.0, 10.0) * rng.uniform(0.6, 1.0, 3)]
        geo = {"type": "triangle_mesh", "filename": "$env{scene_directory}/quad.obj"} if k == 0 else \
            f"$reference{{$root/scene/entities/{instances + 1}/geometry}}"
        ents.append(_entity(geo, _diffuse([0.0, 0.0, 0.0]), [{"scale": [s, 1.0, s]}, {"translate": [float(x), y, float(z)]}],
                            light={"type": "mesh_light", "intensity": inten}))
    scene = {
        "width": width, "height": height,
        "camera": {"type": "pinhole", "eye": [0.0, 0.75, 1.55], "dst": [0.0, 0.0, 0.0], "up": [0.0, 1.0, 0.0],
                   "fov_y": {"deg": 45.0}},
        "renderer": {"type": "wfpt", "spp": spp, "min_depth": 5, "max_depth": 16, "rr_threshold": 0.1,
                     "rr_cont_prob": 0.5, "state_count": state_count, "sampler": "independent",
                     "filter": {"type": "gaussian", "radius": 1.5, "alpha": 1.6}},
        "scene": {"entities": ents,
                  "envir_light": {"type": "gradient_sky", "lower": [0.1, 0.1, 0.12], "upper": [0.6, 0.75, 1.0],
                                  "up": [0.0, 1.0, 0.0]}},
    }
    return _write_scene(out / name, scene)


def random_soup(path_dir: Path, seed: int, n_tris: int, n_instances: int = 3) -> Path:
    """Small traversal-test scene: random triangles in a few translated/scaled instances
    sharing one geometry, plus a ground quad."""
    out = Path(path_dir)
    out.mkdir(parents=True, exist_ok=True)
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1, 1, (n_tris, 3))
    v = c[:, None, :] + rng.normal(0, 0.08, (n_tris, 3, 3))
    write_obj(out / "soup.obj", v.reshape(-1, 3), np.arange(n_tris * 3).reshape(-1, 3))
    qv, qf = quad(4.0)
    write_obj(out / "ground.obj", qv, qf)
    ents = [_entity({"type": "triangle_mesh", "filename": "$env{scene_directory}/ground.obj"}, _diffuse([0.5] * 3),
                    [{"translate": [0.0, -1.5, 0.0]}])]
    for k in range(n_instances):
        geo = {"type": "triangle_mesh", "filename": "$env{scene_directory}/soup.obj"} if k == 0 else \
            "$reference{$root/scene/entities/1/geometry}"
        s = float(rng.uniform(0.5, 1.0))
        t = [float(x) for x in rng.uniform(-1, 1, 3)]
        ents.append(_entity(geo, _diffuse(rng.uniform(0.2, 0.8, 3)), [{"scale": [s, s, s]}, {"translate": t}]))
    scene = {
        "width": 64, "height": 64,
        "camera": {"type": "pinhole", "eye": [0.0, 0.0, 4.0], "dst": [0.0, 0.0, 0.0], "up": [0.0, 1.0, 0.0],
                   "fov_y": {"deg": 50.0}},
        "renderer": {"type": "wfpt", "spp": 4},
        "scene": {"entities": ents},
    }
    return _write_scene(out / "scene.json", scene)


def write_grid(path: Path, grid: np.ndarray) -> None:
    """Binary density grid: b"BTG1", int32 width, height, depth, float32 values (x fastest)."""
    d, h, w = grid.shape
    tmp = path.with_suffix(path.suffix + ".tmp")
    with open(tmp, "wb") as f:
        f.write(b"BTG1")
        f.write(np.array([w, h, d], np.int32).tobytes())
        f.write(np.ascontiguousarray(grid, np.float32).tobytes())
    os.replace(tmp, path)


def write_grid_text(path: Path, grid: np.ndarray) -> None:
    """The reference's text format: "float 1 W H D" then values, x fastest
    (common/btrc/utils/cuda/array.cpp:313-384)."""
    d, h, w = grid.shape
    body = " ".join("%.6g" % v for v in grid.ravel())
    path.write_text(f"float 1 {w} {h} {d}\n{body}\n")


def fbm_grid(perlin: Perlin, res: int, freq: float = 4.0, slab: int = 16) -> np.ndarray:
    """fBm (8 octaves, lacunarity 2) sampled at voxel centres of [0,1]^3, (res, res, res) z-major."""
    out = np.zeros((res, res, res), np.float32)
    c = (np.arange(res) + 0.5) / res
    Y, X = np.meshgrid(c, c, indexing="ij")
    for z0 in range(0, res, slab):
        zs = c[z0:z0 + slab]
        Z = np.broadcast_to(zs[:, None, None], (len(zs), res, res))
        out[z0:z0 + len(zs)] = perlin.fbm3(np.broadcast_to(X, Z.shape) * freq + 0.31,
                                           np.broadcast_to(Y, Z.shape) * freq + 0.17, Z * freq + 0.53, octaves=8)
    return out


def displaced_sphere(perlin: Perlin, level: int, radius: float, amp: float):
    v, f = icosphere(level)
    disp = perlin.fbm3(v[:, 0] * 3 + 11.1, v[:, 1] * 3 + 7.7, v[:, 2] * 3 + 3.3, octaves=4)
    p = v * (radius + amp * disp)[:, None]
    tri = p[f]
    fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    vn = np.zeros_like(p)
    for k in range(3):
        np.add.at(vn, f[:, k], fn)
    vn /= np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-30)
    return p, f, vn


def volume(seed: int = 1002, width: int = 1024, height: int = 1024, spp: int = 64, grid_res: int = 256,
           sphere_level: int = 7, text_grid: bool = False, out_dir: Path | None = None, force: bool = False,
           state_count: int = 32 * 1024 * 1024) -> Path:
    """Config 2: the cornell box with a heterogeneous fBm medium (sigma_t max 20, albedo 0.9,
    HG g 0.6) behind a transform inside an invisible cube, plus a displaced icosphere with a
    GGX conductor of roughness 0.2; depth 32."""
    out = Path(out_dir or cache_dir() / f"volume-{seed}-{grid_res}-{sphere_level}")
    out.mkdir(parents=True, exist_ok=True)
    name = f"scene-{width}x{height}-{spp}-q{state_count}.json"
    if (out / name).exists() and not force:
        return out / name
    rng = np.random.default_rng(seed)
    perlin = Perlin(rng)
    half = 0.5
    bv, bf = box_inward((-half, -half, -half), (half, half, 1.4))
    write_obj(out / "box_left.obj", bv, bf[0:2])
    write_obj(out / "box_right.obj", bv, bf[2:4])
    write_obj(out / "box_rest.obj", bv, bf[4:12])
    qv, qf = quad(0.25)
    write_obj(out / "light.obj", qv, flip(qf))
    ch = 0.475  # medium cube, 5% inside the box cross-section
    cv, cf = box_inward((-ch, -ch, -ch), (ch, ch, ch))
    write_obj(out / "cube.obj", cv, flip(cf))  # normals facing outwards
    sv, sf, sn = displaced_sphere(perlin, sphere_level, 0.22, 0.03)
    write_obj(out / "sphere.obj", sv, sf, normals=sn)
    dens = np.clip(fbm_grid(perlin, grid_res), 0.0, 1.0) * 20.0
    if text_grid:
        write_grid_text(out / "density.txt", dens)
        sigma = {"type": "array", "text": "$env{scene_directory}/density.txt"}
    else:
        write_grid(out / "density.bin", dens)
        sigma = {"type": "array", "binary": "$env{scene_directory}/density.bin"}
    albedos = rng.uniform(0.2, 0.8, (4, 3))
    medium = {"type": "transform", "world_to_local": {"scale": [1.0 / ch] * 3},
              "medium": {"type": "hetergeneous", "sigma_t": sigma, "albedo": 0.9, "g": 0.6}}
    ents = [_entity({"type": "triangle_mesh", "filename": f"$env{{scene_directory}}/{part}.obj"}, _diffuse(albedos[k]))
            for k, part in enumerate(("box_left", "box_right", "box_rest"))]
    ents.append(_entity({"type": "triangle_mesh", "filename": "$env{scene_directory}/light.obj"}, _diffuse(albedos[3]),
                        [{"translate": [0.0, half - 0.005, 0.0]}],
                        light={"type": "mesh_light", "intensity": [15.0, 15.0, 15.0]}))
    ents.append(_entity({"type": "triangle_mesh", "filename": "$env{scene_directory}/cube.obj"}, {"type": "invisible"},
                        inner=medium))
    ents.append(_entity({"type": "triangle_mesh", "filename": "$env{scene_directory}/sphere.obj"},
                        {"type": "metal", "color": [0.95, 0.64, 0.54], "roughness": 0.2},
                        outer="$reference{$root/scene/entities/4/inner_medium}"))
    scene = {
        "width": width, "height": height,
        "camera": {"type": "pinhole", "eye": [0.0, 0.0, 1.3], "dst": [0.0, 0.0, -half], "up": [0.0, 1.0, 0.0],
                   "fov_y": {"deg": 40.0}},
        "renderer": {"type": "wfpt", "spp": spp, "min_depth": 5, "max_depth": 32, "rr_threshold": 0.1,
                     "rr_cont_prob": 0.5, "state_count": state_count, "sampler": "independent",
                     "filter": {"type": "gaussian", "radius": 1.5, "alpha": 1.6}},
        "scene": {"entities": ents},
    }
    return _write_scene(out / name, scene)


def _sphere_uv(level: int):
    """Icosphere with spherical texture coordinates (u from the azimuth, v from the polar
    angle); normals are the positions."""
    v, f = icosphere(level)
    u = np.arctan2(v[:, 2], v[:, 0]) / (2 * np.pi) + 0.5
    t = np.arccos(np.clip(v[:, 1], -1, 1)) / np.pi
    return v, f, np.stack([u, t], 1)


def textured(seed: int = 1003, width: int = 256, height: int = 192, spp: int = 64, out_dir: Path | None = None,
             force: bool = False, lut: tuple[int, int] = (64, 32)) -> Path:
    """Image textures, texture expressions, normal maps and an HDR environment light:
    a checker-textured, bump-mapped ground (sRGB PNG, wrap / mirror addressing), a Disney
    sphere whose colour is a palette PNG times a constant and whose roughness is a rotated,
    scaled 16-bit PNG, a metal sphere with a 4-bit border-addressed roughness map plus a
    constant, and a glass sphere with a constant normal map, all lit by an `ibl` light over
    a run-length-encoded Radiance HDR sky (builtin/btrc/builtin/light/ibl.cpp)."""
    out = Path(out_dir or cache_dir() / f"textured-{seed}")
    out.mkdir(parents=True, exist_ok=True)
    name = f"scene-{width}x{height}-{spp}-{lut[0]}x{lut[1]}.json"
    if (out / name).exists() and not force:
        return out / name
    rng = np.random.default_rng(seed)
    # textures
    yy, xx = np.mgrid[0:64, 0:64]
    chk = ((xx // 8 + yy // 8) % 2).astype(np.float64)
    c0, c1 = rng.uniform(0.1, 0.4, 3), rng.uniform(0.6, 0.95, 3)
    rgb = chk[..., None] * c1 + (1 - chk[..., None]) * c0 + rng.uniform(-0.03, 0.03, (64, 64, 3))
    write_png(out / "checker.png", np.clip(rgb * 255, 0, 255).astype(np.uint8))
    hy, hx = np.mgrid[0:32, 0:32] / 32.0
    hgt = 0.5 * np.sin(2 * np.pi * 3 * hx) * np.cos(2 * np.pi * 2 * hy)
    gx, gy = np.gradient(hgt, 1 / 32.0)
    nrm = np.stack([-gx * 0.05, -gy * 0.05, np.ones_like(hgt)], -1)
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    rgba = np.concatenate([(nrm * 0.5 + 0.5) * 255, np.full((32, 32, 1), 255.0)], -1)
    write_png(out / "bumps.png", np.clip(rgba, 0, 255).astype(np.uint8))
    pal = rng.integers(30, 255, (8, 3))
    write_png(out / "palette.png", rng.integers(0, 8, (16, 16)), palette=pal, alpha=[255, 200, 255, 128])
    write_png(out / "rough16.png", rng.integers(5000, 60000, (32, 32)), depth=16)
    write_png(out / "rough4.png", rng.integers(0, 16, (16, 16)), depth=4)
    ey, ex = np.mgrid[0:64, 0:128]
    theta = (ey + 0.5) / 64 * np.pi
    phi = (ex + 0.5) / 128 * 2 * np.pi
    sky = np.stack([0.3 + 0.5 * np.cos(theta).clip(0), 0.45 + 0.5 * np.cos(theta).clip(0), 0.7 + 0.4 * np.cos(theta).clip(0)], -1)
    sky[theta > np.pi / 2] = [0.12, 0.1, 0.08]
    sun = np.exp(-((theta - 0.6) ** 2 + (phi - 1.3) ** 2) / 0.01)
    sky += sun[..., None] * np.array([60.0, 55.0, 45.0])
    write_hdr(out / "sky.hdr", sky)
    # geometry
    qv = np.array([[-2, 0, -2], [2, 0, -2], [2, 0, 2], [-2, 0, 2]], np.float64)
    qf = np.array([[0, 2, 1], [0, 3, 2]], np.int64)
    quv = np.array([[0, 0], [3, 0], [3, 3], [0, 3]], np.float64)
    write_obj(out / "ground.obj", qv, qf, normals=np.tile([[0, 1, 0]], (4, 1)), uvs=quv)
    sv, sf, suv = _sphere_uv(4)
    write_obj(out / "sphere_uv.obj", sv, sf, normals=sv, uvs=suv)

    def arr(fn, **kw):
        d = {"type": "array", "filename": "$env{scene_directory}/" + fn}
        d.update(kw)
        return d
    ents = [
        _entity({"type": "triangle_mesh", "filename": "$env{scene_directory}/ground.obj"},
                {"type": "diffuse",
                 "color": arr("checker.png", srgb_to_linear=True, address_mode_u="wrap", address_mode_v="mirror"),
                 "normal": arr("bumps.png", address_mode_u="wrap", address_mode_v="wrap")},
                [{"translate": [0.0, -0.3, 0.0]}]),
        _entity({"type": "triangle_mesh", "filename": "$env{scene_directory}/sphere_uv.obj"},
                {"type": "disney",
                 "color": {"type": "mul", "lhs": arr("palette.png", filter="point", address_mode_u="wrap"),
                           "rhs": [0.9, 0.85, 0.8]},
                 "metallic": 0.0,
                 "roughness": {"type": "transform", "transform": [{"scale": [2, 2]}, {"rotate": {"angle": {"deg": 30}}}],
                               "tex": arr("rough16.png", address_mode_u="wrap", address_mode_v="wrap")},
                 "clearcoat": 0.3},
                [{"scale": [0.3, 0.3, 0.3]}, {"translate": [-0.7, 0.0, 0.0]}]),
        _entity({"type": "triangle_mesh", "filename": "$env{scene_directory}/sphere_uv.obj"},
                {"type": "metal", "color": [0.9, 0.7, 0.5],
                 "roughness": {"type": "add", "lhs": arr("rough4.png", address_mode_u="border", address_mode_v="border",
                                                          border=0.2),
                               "rhs": 0.05}},
                [{"scale": [0.3, 0.3, 0.3]}]),
        _entity({"type": "triangle_mesh", "filename": "$env{scene_directory}/sphere_uv.obj"},
                {"type": "glass", "color": [1.0, 1.0, 1.0], "ior": 1.5, "normal": [0.5, 0.5, 1.0]},
                [{"scale": [0.3, 0.3, 0.3]}, {"translate": [0.7, 0.0, 0.0]}]),
    ]
    scene = {
        "width": width, "height": height,
        "camera": {"type": "pinhole", "eye": [0.0, 0.45, 2.2], "dst": [0.0, -0.05, 0.0], "up": [0.0, 1.0, 0.0],
                   "fov_y": {"deg": 40.0}},
        "renderer": {"type": "wfpt", "spp": spp, "min_depth": 3, "max_depth": 8, "rr_threshold": 0.1,
                     "rr_cont_prob": 0.5, "state_count": 1000000, "sampler": "halton",
                     "filter": {"type": "gaussian", "radius": 1.5, "alpha": 1.6}},
        "scene": {"entities": ents,
                  "envir_light": {"type": "ibl", "tex": arr("sky.hdr", address_mode_u="wrap"), "up": [0.0, 1.0, 0.0],
                                  "lut_width": lut[0], "lut_height": lut[1]}},
    }
    _write_scene(out / name, scene)
    return out / name


def _write_terrain_mesh(path: Path, perlin: Perlin, grid: int) -> None:
    xs = np.linspace(-1.0, 1.0, grid)
    X, Z = np.meshgrid(xs, xs, indexing="xy")
    H = 0.2 * perlin.fbm3(X * 2.0 + 0.5, Z * 2.0 + 0.5, np.full_like(X, 0.37), octaves=8, lacunarity=2.0)
    V = np.stack([X, H, Z], axis=-1).reshape(-1, 3)
    dhdx = np.gradient(H, xs, axis=1)
    dhdz = np.gradient(H, xs, axis=0)
    N = np.stack([-dhdx, np.ones_like(H), -dhdz], axis=-1)
    N /= np.linalg.norm(N, axis=-1, keepdims=True)
    idx = np.arange(grid * grid).reshape(grid, grid)
    a, b, c, d = idx[:-1, :-1], idx[:-1, 1:], idx[1:, :-1], idx[1:, 1:]
    F = np.concatenate([np.stack([a, c, b], -1).reshape(-1, 3), np.stack([b, c, d], -1).reshape(-1, 3)])
    write_obj(path, V, F, normals=N.reshape(-1, 3))


def batch(count: int = 64, seed: int = 1004, out_dir: Path | None = None, force: bool = False) -> list[Path]:
    """Batched uneven scenes: `count` seeded terrain scenes in the style of the large-mesh
    scene (fBm heightfield, instanced spheres, Disney materials, 8 quad lights and a sky),
    triangle counts log-uniform in [1e4, 5e5] (eight shared meshes, one per octave step),
    films of 128^2, 256^2, 384^2 or 512^2, 16, 32 or 64 spp, depth 12."""
    out = Path(out_dir or cache_dir() / f"batch-{seed}-{count}")
    out.mkdir(parents=True, exist_ok=True)
    rng = np.random.default_rng(seed)
    perlin = Perlin(rng)
    levels = [1e4 * 50 ** (k / 7) for k in range(8)]
    grids = [int(round(np.sqrt(t / 2))) for t in levels]
    for k, g in enumerate(grids):
        if force or not (out / f"terrain{k}.obj").exists():
            _write_terrain_mesh(out / f"terrain{k}.obj", perlin, g + 1)
    if force or not (out / "sphere2.obj").exists():
        sv, sf = icosphere(2)
        write_obj(out / "sphere2.obj", sv, sf, normals=sv)
        qv, qf = quad(1.0)
        write_obj(out / "quad.obj", qv, flip(qf))
    paths = []
    for i in range(count):
        r = np.random.default_rng(seed * 1000 + i)
        k = int(r.integers(0, 8))
        res = int(r.choice([128, 256, 384, 512]))
        spp = int(r.choice([16, 32, 64]))
        name = out / f"scene{i:03d}.json"
        paths.append(name)
        if name.exists() and not force:
            continue

        def disney():
            return {"type": "disney", "color": [float(v) for v in r.uniform(0, 1, 3)],
                    "roughness": float(r.uniform(0.05, 1.0)), "metallic": float(r.random() < 0.3),
                    "specular": 0.5, "clearcoat": float(r.uniform(0, 1))}
        ents = [_entity({"type": "triangle_mesh", "filename": f"$env{{scene_directory}}/terrain{k}.obj"}, disney())]
        for j in range(8):
            x, z = r.uniform(-0.9, 0.9, 2)
            s = float(r.uniform(0.02, 0.06))
            geo = {"type": "triangle_mesh", "filename": "$env{scene_directory}/sphere2.obj"} if j == 0 else \
                "$reference{$root/scene/entities/1/geometry}"
            ents.append(_entity(geo, disney(), [{"scale": [s, s, s]}, {"translate": [float(x), 0.25, float(z)]}]))
        for j in range(8):
            x, z = r.uniform(-0.8, 0.8, 2)
            s = float(r.uniform(0.05, 0.15))
            inten = [float(v) for v in r.uniform(2.0, 10.0) * r.uniform(0.6, 1.0, 3)]
            geo = {"type": "triangle_mesh", "filename": "$env{scene_directory}/quad.obj"} if j == 0 else \
                "$reference{$root/scene/entities/9/geometry}"
            ents.append(_entity(geo, _diffuse([0.0, 0.0, 0.0]), [{"scale": [s, 1.0, s]},
                                                                  {"translate": [float(x), 0.5, float(z)]}],
                                light={"type": "mesh_light", "intensity": inten}))
        ang = float(r.uniform(0, 2 * np.pi))
        scene = {
            "width": res, "height": res,
            "camera": {"type": "pinhole", "eye": [1.6 * np.sin(ang), 0.8, 1.6 * np.cos(ang)], "dst": [0.0, 0.0, 0.0],
                       "up": [0.0, 1.0, 0.0], "fov_y": {"deg": 45.0}},
            "renderer": {"type": "wfpt", "spp": spp, "min_depth": 5, "max_depth": 12, "rr_threshold": 0.1,
                         "rr_cont_prob": 0.5, "state_count": 1 << 20, "sampler": "independent",
                         "filter": {"type": "gaussian", "radius": 1.5, "alpha": 1.6}},
            "scene": {"entities": ents,
                      "envir_light": {"type": "gradient_sky", "lower": [0.1, 0.1, 0.12], "upper": [0.6, 0.75, 1.0],
                                      "up": [0.0, 1.0, 0.0]}},
        }
        _write_scene(name, scene)
    return paths
