"""Two-level acceleration structure (btrc_build_opts.two_level): per-geometry object-space
trees under a top-level tree over instance boxes, the form of the reference's OptiX IAS
over GASes (core/btrc/core/scene.cpp:196-209).

- traversal: closest hit (flags, t, barycentrics) and any hit bit-exact against the
  oracle's two-level restatement (oracle.two_level_trace: the same rounded object-space
  rays, the oracle's own watertight test, hits combined in (t, instance, primitive)
  order), on random rays, segments, rays from hundreds of scene sizes away and rays
  aimed at triangle vertices and edges;
- memory: the two-level scene holds each instanced geometry once;
- rendering: a frame through the two-level form equals the flattened form's frame up to
  the rounding of object-space hit distances."""
import numpy as np
import pytest

import oracle
from btrc_gb300 import scenes
from oracle import scene as OS
from tests.test_gpu_trace import _gpu_trace
from tests.util import edge_rays, rel_mse

pytestmark = pytest.mark.gpu


def _rays(rng, S, n, n_edge):
    rays = np.zeros((n, 8), np.float32)
    lo, hi = S.tris.reshape(-1, 3).min(0), S.tris.reshape(-1, 3).max(0)
    rays[:, 0:3] = rng.uniform(lo - 0.5, hi + 0.5, (n, 3))
    rays[:, 4:7] = rng.normal(size=(n, 3))
    rays[:, 7] = 3.0e38
    seg = rng.random(n) < 0.3
    rays[seg, 4:7] *= rng.uniform(0.05, 2.0, (int(seg.sum()), 1)).astype(np.float32)
    rays[seg, 7] = 1.0
    # far origins (hundreds of scene sizes away) aimed at triangle centroids: box tests
    # must stay conservative when distances dwarf the instance boxes' padding
    m = n // 10
    tgt = S.tris[rng.integers(0, len(S.tris), m)].reshape(m, 3, 3).mean(1)
    d = rng.normal(size=(m, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    far = np.zeros((m, 8), np.float32)
    far[:, 0:3] = tgt - d * rng.uniform(100.0, 1000.0, (m, 1)) * float(np.max(hi - lo))
    far[:, 4:7] = d
    far[:, 7] = 3.0e38
    return np.concatenate([rays, far, edge_rays(rng, S.tris, n_edge)])


def _compare(ctx, path, n=20000, n_edge=10000, seed=3):
    S = OS.Scene(path)
    rays = _rays(np.random.default_rng(seed), S, n, n_edge)
    sc = ctx.load_scene(path).build(two_level=True)
    assert sc.info().two_level == 1
    g_flags, g_hits, g_occ = _gpu_trace(ctx, sc, rays)
    o_flags, o_hits, o_occ = oracle.two_level_trace(S, rays)
    bad = np.nonzero(g_flags != o_flags)[0]
    assert len(bad) == 0, f"{len(bad)} flag mismatches, first {bad[:5]}: gpu {g_flags[bad[:5]]} oracle {o_flags[bad[:5]]}"
    hit = o_flags != 0
    assert np.array_equal(g_hits[hit].view(np.uint32), o_hits[hit].view(np.uint32))
    assert np.array_equal(g_occ, o_occ)
    assert 0.05 < hit.mean()
    return sc, hit


@pytest.mark.parametrize("which", ["soup", "terrain", "cornell"])
def test_two_level_traversal_bitexact(gpu_ctx, scene_dir, which):
    if which == "soup":
        path = scenes.random_soup(scene_dir / "soup", seed=5, n_tris=20000, n_instances=4)
    elif which == "cornell":
        path = scenes.cornell(out_dir=scene_dir / "cornell")
    else:
        path = scenes.terrain(seed=7, width=64, height=64, spp=1, grid=128, instances=8,
                              out_dir=scene_dir / "terrain")
    _compare(gpu_ctx, path)


def test_two_level_bench_terrain(gpu_ctx, scene_dir):
    """The benchmark terrain (2.1 M-triangle heightfield and 200 instances of one 5120-
    triangle icosphere): bit-exact against the oracle, and the two-level form holds the
    icosphere once instead of 200 times."""
    path = scenes.terrain(width=1920, height=1080, spp=16, out_dir=scene_dir / "terrain-bench")
    sc, hit = _compare(gpu_ctx, path, n=20000, n_edge=5000, seed=21)
    flat = gpu_ctx.load_scene(path).build()
    two, one = sc.info(), flat.info()
    assert two.triangles == one.triangles == 3117074
    # 2.1 M + 5120 triangle records against 3.1 M
    assert two.bvh_bytes < 0.75 * one.bvh_bytes, (two.bvh_bytes, one.bvh_bytes)


def test_two_level_render_matches_flattened(gpu_ctx, scene_dir):
    path = scenes.terrain(seed=7, width=64, height=64, spp=16, grid=128, instances=8, out_dir=scene_dir / "terrain-r")
    two = gpu_ctx.load_scene(path).build(two_level=True)
    flat = gpu_ctx.load_scene(path).build()
    a = gpu_ctx.render(two)
    b = gpu_ctx.render(flat)
    # same sampler streams; object-space hit distances differ from world-space ones in
    # the last bits, which moves hit points by rounding amounts only
    assert rel_mse(a, b) < 1e-4


def test_two_level_refused_by_merged_batch(gpu_ctx, scene_dir):
    import btrc_gb300 as B
    path = scenes.random_soup(scene_dir / "soup", seed=5, n_tris=2000, n_instances=2)
    sc = gpu_ctx.load_scene(path).build(two_level=True)
    out = np.zeros((64, 64, 3), np.float32)
    with pytest.raises(B.BtrcError) as e:
        gpu_ctx.render_batch([sc], [out], merged=True)
    assert e.value.status == 8


def test_two_level_noalloc_and_cache_frames(gpu_ctx, scene_dir):
    """The allocation-free entry point and the radiance-cache frames (whose training paths
    walk the two-level form one thread per path) take two-level scenes too."""
    import torch
    import btrc_gb300 as B
    path = scenes.terrain(seed=7, width=64, height=64, spp=4, grid=128, instances=8, out_dir=scene_dir / "terrain-n")
    sc = gpu_ctx.load_scene(path).build(two_level=True)
    ref = gpu_ctx.render(sc)
    out = torch.zeros((64, 64, 3), dtype=torch.float32, device="cuda")
    gpu_ctx.render_noalloc(sc, out)
    torch.cuda.synchronize()
    assert np.allclose(out.cpu().numpy(), ref, rtol=1e-5, atol=1e-6)
    info = sc.info()
    cache = B.RadianceCache(gpu_ctx, info.world_min, info.world_max, seed=1)
    st = {}
    img = cache.render_frame(sc, 0, stats=st)
    cache.render_frame(sc, 1, stats=st)
    assert np.all(np.isfinite(img)) and st["train_samples"] > 0 and st["queries"] > 0
    cache.close()

