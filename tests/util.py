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
