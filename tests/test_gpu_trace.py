"""Closest-hit and any-hit traversal on the GPU, bit-exact against the oracle.

Bar: identical flag words (instance | hit bit), primitive ids, t, b1, b2 bits for every
ray; exact ties in t resolve to the lower (instance, primitive) on both sides."""
import numpy as np
import pytest

import oracle
from btrc_gb300 import scenes
from oracle import scene as OS
from tests.util import edge_rays, random_rays

pytestmark = pytest.mark.gpu


def _gpu_trace(ctx, sc, rays):
    import torch
    n = len(rays)
    d_rays = torch.from_numpy(np.ascontiguousarray(rays)).cuda()
    flags = torch.zeros(n, dtype=torch.int32, device="cuda")
    hits = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    occ = torch.zeros(n, dtype=torch.int32, device="cuda")
    ctx.trace_closest(sc, d_rays, n, flags, hits)
    ctx.trace_any(sc, d_rays, n, occ)
    torch.cuda.synchronize()
    return flags.cpu().numpy().view(np.uint32), hits.cpu().numpy(), occ.cpu().numpy().view(np.uint32)


def _compare(ctx, path, rays):
    sc = ctx.load_scene(path).build()
    S = OS.Scene(path)
    g_flags, g_hits, g_occ = _gpu_trace(ctx, sc, rays)
    bvh = oracle.OracleBvh(S.tris, S.ids)
    o_flags, o_hits = bvh.closest(rays)
    o_occ = bvh.any(rays)
    bad = np.nonzero(g_flags != o_flags)[0]
    assert len(bad) == 0, f"{len(bad)} flag mismatches, first {bad[:5]}: gpu {g_flags[bad[:5]]} oracle {o_flags[bad[:5]]}"
    hit = o_flags != 0
    assert np.array_equal(g_hits[hit].view(np.uint32), o_hits[hit].view(np.uint32))
    assert np.array_equal(g_occ, o_occ)
    # any-hit agrees with closest-hit existence
    assert np.array_equal(g_occ != 0, g_flags != 0)
    return sc, hit.mean()


def test_closest_bitexact_cornell(gpu_ctx, scene_dir):
    p = scenes.cornell(out_dir=scene_dir / "cornell")
    rng = np.random.default_rng(11)
    inside = random_rays(rng, 200000, -0.45, 0.45)
    S = OS.Scene(p)
    rays = np.concatenate([inside, edge_rays(rng, S.tris, 50000)])
    sc, _ = _compare(gpu_ctx, p, rays)
    # every ray that starts inside the closed box hits a wall
    f, _, _ = _gpu_trace(gpu_ctx, sc, inside)
    assert (f != 0).all()


def test_closest_bitexact_instanced_soup(gpu_ctx, scene_dir):
    p = scenes.random_soup(scene_dir / "soup", seed=5, n_tris=20000, n_instances=4)
    rng = np.random.default_rng(12)
    S = OS.Scene(p)
    rays = np.concatenate([random_rays(rng, 200000, -2.0, 2.0), edge_rays(rng, S.tris, 100000)])
    _compare(gpu_ctx, p, rays)


def test_t1_limits_and_shadow_segments(gpu_ctx, scene_dir):
    # finite t1 (area-light shadow rays use t1 = 1 with an unnormalised direction)
    p = scenes.random_soup(scene_dir / "soup", seed=5, n_tris=20000, n_instances=4)
    rng = np.random.default_rng(13)
    rays = random_rays(rng, 200000, -2.0, 2.0, t1=1.0)
    rays[:, 4:7] *= rng.uniform(0.05, 3.0, (len(rays), 1)).astype(np.float32)
    _compare(gpu_ctx, p, rays)


def test_empty_batch_and_misses(gpu_ctx, scene_dir):
    import torch
    p = scenes.random_soup(scene_dir / "soup", seed=5, n_tris=2000, n_instances=1)
    sc = gpu_ctx.load_scene(p).build()
    # n == 0 is a no-op
    gpu_ctx.trace_closest(sc, None, 0, None, None)
    gpu_ctx.trace_any(sc, None, 0, None)
    # rays pointing away from everything miss; flags 0, detail zeroed
    rays = np.zeros((1000, 8), np.float32)
    rays[:, 0:3] = [0.0, 50.0, 0.0]
    rays[:, 4:7] = [0.0, 1.0, 0.0]
    rays[:, 7] = 3.0e38
    f, h, o = _gpu_trace(gpu_ctx, sc, rays)
    assert (f == 0).all() and (o == 0).all() and (h == 0).all()


def test_invalid_arguments(gpu_ctx, scene_dir):
    import btrc_gb300 as B
    p = scenes.random_soup(scene_dir / "soup", seed=5, n_tris=2000, n_instances=1)
    sc = gpu_ctx.load_scene(p)
    with pytest.raises(B.BtrcError) as e:
        gpu_ctx.trace_closest(sc, 1, 1, 1, 1)  # not built
    assert e.value.status == 1


def test_closest_bitexact_small_terrain(gpu_ctx, scene_dir):
    # a 128^2 heightfield with 8 instanced spheres (~73 K triangles): the 8-wide nodes of
    # the dynamic-programming collapse are mostly full, leaves hold 1-3 triangles, and rays
    # from above graze the surface at every angle
    p = scenes.terrain(seed=7, width=64, height=64, spp=1, grid=128, instances=8, out_dir=scene_dir / "terrain")
    rng = np.random.default_rng(14)
    S = OS.Scene(p)
    n = 100000
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform([-1.2, 0.3, -1.2], [1.2, 1.5, 1.2], (n, 3))
    d = rng.normal(size=(n, 3))
    d[:, 1] = -np.abs(d[:, 1]) * rng.uniform(0.05, 1.0, n)
    rays[:, 4:7] = d
    rays[:, 7] = 3.0e38
    rays = np.concatenate([rays, edge_rays(rng, S.tris, 50000)])
    _, hit_rate = _compare(gpu_ctx, p, rays)
    assert hit_rate > 0.25


def test_kernel_counts_match_oracle_traversal(gpu_ctx, scene_dir):
    """The closest-hit kernel's per-ray work counters (btrc_trace_stats) against the
    oracle's sequential exact-box traversal of the same BVH: the kernel's padded FP32 box
    tests can only add visits, and only a few percent of them."""
    import torch
    import btrc_gb300 as B
    path = scenes.random_soup(scene_dir / "soup", seed=5, n_tris=20000, n_instances=4)
    hctx = B.Context(-1)
    hsc = hctx.load_scene(path).build()
    nodes, tris = hsc.export_bvh()
    sc = gpu_ctx.load_scene(path).build()
    rng = np.random.default_rng(10)
    n = 20000
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(-2, 2, (n, 3))
    rays[:, 4:7] = rng.normal(size=(n, 3))
    rays[:, 7] = 3.0e38
    nv, tt = oracle.wide_bvh_counts(nodes, tris, rays)
    dr = torch.from_numpy(rays).cuda()
    gn = torch.zeros(n, dtype=torch.int32, device="cuda")
    gt = torch.zeros(n, dtype=torch.int32, device="cuda")
    gpu_ctx.trace_stats(sc, dr, n, gn, gt)
    torch.cuda.synchronize()
    gn, gt = gn.cpu().numpy(), gt.cpu().numpy()
    assert gn.mean() >= nv.mean() * 0.999 and gn.mean() <= nv.mean() * 1.05, (gn.mean(), nv.mean())
    assert gt.mean() >= tt.mean() * 0.999 and gt.mean() <= tt.mean() * 1.05, (gt.mean(), tt.mean())
    sc.close()
    hsc.close()
    hctx.close()
