"""Writes the lib/bvh golden fixtures of this folder.

The reference tree vendors a CPU BVH library (lib/bvh: SweepSahBuilder, SingleRayTraverser,
ClosestPrimitiveIntersector). `oracle/build.py` compiles a small driver around it from the
reference sources into `oracle/_ref/` when the reference tree is present; this script runs
that driver on fixed, seeded triangle sets and rays and stores its closest hits (flat
primitive index, t), so that the oracle's traversal stays pinned to the reference's own
code on machines without the reference tree.

Run from the repository root:  python tests/golden/make_lib_bvh_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from btrc_gb300 import scenes  # noqa: E402
from oracle import scene as OS  # noqa: E402

OUT = Path(__file__).resolve().parent


def _write(name, tris, ids, rays):
    res = oracle.ref_closest(tris, rays)
    if res is None:
        raise SystemExit("lib/bvh driver not built (oracle/_ref): run oracle/build.py with the reference tree present")
    prim, t = res
    np.savez_compressed(OUT / name, tris=tris.astype(np.float32), ids=ids.astype(np.uint32),
                        rays=rays.astype(np.float32), prim=prim.astype(np.int64), t=t.astype(np.float32))
    print(f"{name}: {len(tris)} triangles, {len(rays)} rays, hit rate {(prim >= 0).mean():.3f}")


def main():
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        # config 0's Cornell box: rays from inside the closed box in every direction
        S = OS.Scene(scenes.cornell(out_dir=Path(d)))
        rng = np.random.default_rng(1701)
        n = 8000
        rays = np.zeros((n, 8), np.float32)
        rays[:, 0:3] = rng.uniform(-0.45, 0.45, (n, 3))
        rays[:, 4:7] = rng.normal(size=(n, 3))
        rays[:, 7] = 3.0e38
        _write("lib_bvh_cornell.npz", S.tris, S.ids, rays)
    # a seeded soup of 4000 small triangles in the unit cube, rays from outside and inside
    rng = np.random.default_rng(1702)
    m = 4000
    c = rng.uniform(-1.0, 1.0, (m, 1, 3))
    tris = (c + rng.normal(scale=0.08, size=(m, 3, 3))).reshape(m, 9).astype(np.float32)
    ids = np.stack([np.zeros(m, np.uint32), np.arange(m, dtype=np.uint32)], 1)
    n = 8000
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(-1.6, 1.6, (n, 3))
    rays[:, 4:7] = -rays[:, 0:3] + rng.normal(scale=0.5, size=(n, 3))
    rays[:, 7] = 3.0e38
    _write("lib_bvh_soup.npz", tris, ids, rays)


if __name__ == "__main__":
    main()
