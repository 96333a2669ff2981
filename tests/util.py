"""Shared helpers for the parity tests."""
from __future__ import annotations

import numpy as np


def random_rays(rng, n, lo, hi, t1=3.0e38):
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(lo, hi, (n, 3))
    rays[:, 4:7] = rng.normal(size=(n, 3))
    rays[:, 7] = t1
    return rays


def edge_rays(rng, tris, n, t1=3.0e38):
    """Rays aimed exactly at triangle vertices and edge midpoints (watertightness cases),
    plus axis-aligned directions (zero direction components)."""
    idx = rng.integers(0, len(tris), n)
    t = tris[idx].reshape(n, 3, 3).astype(np.float64)
    which = rng.integers(0, 6, n)
    tgt = np.where((which < 3)[:, None], t[np.arange(n), which % 3], 0.5 * (t[np.arange(n), which % 3] + t[np.arange(n), (which + 1) % 3]))
    o = tgt + rng.normal(size=(n, 3)) * 0.7
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 4:7] = (tgt - o)
    rays[:, 7] = t1
    # a quarter of them axis aligned
    k = n // 4
    ax = rng.integers(0, 3, k)
    d = np.zeros((k, 3), np.float32)
    d[np.arange(k), ax] = np.where(rng.random(k) < 0.5, -1.0, 1.0)
    rays[:k, 4:7] = d
    return rays


def flatten_index(ids, flags, prims):
    cnt = np.bincount(ids[:, 0])
    offs = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    inst = flags & ((1 << 29) - 1)
    return np.where(flags != 0, offs[inst] + prims, -1)


def rel_mse(img, ref):
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


# A density grid linear in each index: trilinear filtering reproduces it exactly, so along
# any segment inside the filtered range the optical depth is length * sigma(midpoint).
RAMP_RES = (16, 8, 12)
RAMP_COEF = (0.5, 0.2, 0.15, 0.1)   # sigma = a + bx i + by j + bz k at texel (i, j, k)


def ramp_medium_scene(tmp):
    """Write a unit cube of `invisible` material whose inner medium is the linear-ramp
    grid behind a transform medium (world [-0.5, 0.5]^3 -> local [-1, 1]^3 -> uvw
    [0, 1]^3). Returns the scene path; the medium is id 0."""
    import json
    from btrc_gb300 import scenes
    rx, ry, rz = RAMP_RES
    a, bx, by, bz = RAMP_COEF
    k, j, i = np.meshgrid(np.arange(rz), np.arange(ry), np.arange(rx), indexing="ij")
    scenes.write_grid_text(tmp / "ramp.txt", (a + bx * i + by * j + bz * k).astype(np.float32))
    cv, cf = scenes.box_inward((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5))
    scenes.write_obj(tmp / "cube.obj", cv, scenes.flip(cf))
    medium = {"type": "transform", "world_to_local": {"scale": [2, 2, 2]},
              "medium": {"type": "hetergeneous", "albedo": 0.8, "g": 0.0,
                         "sigma_t": {"type": "array", "text": "$env{scene_directory}/ramp.txt"}}}
    scene = {"width": 8, "height": 8,
             "camera": {"type": "pinhole", "eye": [0, 0, 3], "dst": [0, 0, 0], "up": [0, 1, 0], "fov_y": {"deg": 30}},
             "renderer": {"type": "wfpt", "spp": 1},
             "scene": {"entities": [{"geometry": {"type": "triangle_mesh", "filename": "$env{scene_directory}/cube.obj"},
                                     "material": {"type": "invisible"}, "inner_medium": medium}]}}
    p = tmp / "ramp.json"
    p.write_text(json.dumps(scene))
    return p


def ramp_sigma(x):
    """sigma at world points x (..., 3) inside the filtered range |x| <= 0.5 - 0.5 / res:
    uvw = 0.5 + x, texel coordinate = res * uvw - 0.5 (the clamp-addressed trilinear fetch)."""
    a, bx, by, bz = RAMP_COEF
    rx, ry, rz = RAMP_RES
    return (a + bx * (rx * (0.5 + x[..., 0]) - 0.5) + by * (ry * (0.5 + x[..., 1]) - 0.5)
            + bz * (rz * (0.5 + x[..., 2]) - 0.5))


def ramp_segments(seed=3, count=6):
    """Segments (count, 6) with both ends inside the filtered range of every axis."""
    return np.random.default_rng(seed).uniform(-0.43, 0.43, (count, 6))


def ramp_tr_exact(seg):
    a, b = seg[..., :3], seg[..., 3:]
    return np.exp(-np.linalg.norm(b - a, axis=-1) * ramp_sigma(0.5 * (a + b)))
