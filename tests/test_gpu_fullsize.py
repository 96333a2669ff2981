"""Parity at the benchmark's own size: the 1080p terrain (1024^2-vertex heightfield, 200
instanced icospheres, 8 quad lights, sky; 3.12 M triangles, BVH larger than L2).

- traversal: closest hit and any hit bit-exact against the oracle's own BVH on rays from
  above the terrain, rays aimed at triangle vertices and edges, and finite segments;
- rendering: the whole 1920x1080 frame rendered through the wavefront (multi-wave queue,
  captured bounce graphs, second shadow stream), compared on a band of rows with the
  oracle renderer, which follows the same sampler streams (paths coincide)."""
import numpy as np
import pytest

import oracle
from btrc_gb300 import scenes
from oracle import scene as OS
from tests.util import edge_rays, rel_mse

pytestmark = pytest.mark.gpu

WIDTH, HEIGHT, SPP = 1920, 1080, 16


@pytest.fixture(scope="module")
def bench_terrain(scene_dir):
    p = scenes.terrain(width=WIDTH, height=HEIGHT, spp=SPP, out_dir=scene_dir / "terrain-bench")
    return p, OS.Scene(p)


def test_bench_terrain_traversal_bitexact(gpu_ctx, bench_terrain):
    from tests.test_gpu_trace import _gpu_trace
    p, S = bench_terrain
    assert len(S.tris) == 3117074
    rng = np.random.default_rng(21)
    n = 100000
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform([-1.2, 0.3, -1.2], [1.2, 1.5, 1.2], (n, 3))
    d = rng.normal(size=(n, 3))
    d[:, 1] = -np.abs(d[:, 1]) * rng.uniform(0.02, 1.0, n)
    rays[:, 4:7] = d
    rays[:, 7] = 3.0e38
    # a third become segments (shadow-ray form: t1 = 1 with a scaled direction)
    seg = rng.random(n) < 0.33
    rays[seg, 4:7] *= rng.uniform(0.05, 2.0, (int(seg.sum()), 1)).astype(np.float32)
    rays[seg, 7] = 1.0
    rays = np.concatenate([rays, edge_rays(rng, S.tris, 50000)])
    sc = gpu_ctx.load_scene(p).build()
    g_flags, g_hits, g_occ = _gpu_trace(gpu_ctx, sc, rays)
    bvh = oracle.OracleBvh(S.tris, S.ids)
    o_flags, o_hits = bvh.closest(rays)
    o_occ = bvh.any(rays)
    bad = np.nonzero(g_flags != o_flags)[0]
    assert len(bad) == 0, f"{len(bad)} flag mismatches, first {bad[:5]}"
    hit = o_flags != 0
    assert np.array_equal(g_hits[hit].view(np.uint32), o_hits[hit].view(np.uint32))
    assert np.array_equal(g_occ, o_occ)
    assert 0.2 < hit.mean() < 0.9
    # instances are hit too, not only the heightfield (instance 0)
    assert len(np.unique(g_flags[hit] & 0x7fffffff)) > 20


def test_bench_terrain_frame_matches_oracle_band(gpu_ctx, bench_terrain):
    p, S = bench_terrain
    sc = gpu_ctx.load_scene(p).build()
    stats = {}
    g = gpu_ctx.render(sc, spp=SPP, stats=stats).astype(np.float64)
    assert stats["paths"] == WIDTH * HEIGHT * SPP
    assert stats["traversal_errors"] == 0
    assert np.isfinite(g).all()
    # rows 480..575: the horizon band (terrain, instances, sky and lights in view)
    r0, r1, batches = 480, 576, 4
    per = SPP // batches
    films = [S.render(spp=per, sample_begin=k * per, pixel_begin=r0 * WIDTH, pixel_end=r1 * WIDTH)[r0:r1]
             for k in range(batches)]
    imgs = np.stack([OS.resolve(f) for f in films])
    o = imgs.mean(0)
    var = imgs.var(0, ddof=1) / batches
    gb = g[r0:r1]
    err = rel_mse(gb, o)
    assert err < 1e-3, err
    z = np.mean((gb - o) ** 2 / (2 * var + 1e-8))
    assert z < 2.0, z


def test_cornell_config_at_its_own_size(gpu_ctx, scene_dir):
    """The small Cornell workload exactly as specified: 256x256, 16 spp, Halton sampler,
    Gaussian filter importance sampling (radius 1.5), depth 8 with Russian roulette from
    depth 3; the whole image against the oracle renderer on the same sampler streams."""
    p = scenes.cornell(out_dir=scene_dir / "cornell-c0", width=256, height=256, spp=16)
    sc = gpu_ctx.load_scene(p).build()
    info = sc.info()
    assert (info.width, info.height, info.spp, info.sampler, info.filter, info.max_depth) == (256, 256, 16, 1, 1, 8)
    stats = {}
    g = gpu_ctx.render(sc, stats=stats).astype(np.float64)
    assert stats["paths"] == 256 * 256 * 16 and stats["traversal_errors"] == 0
    S = OS.Scene(p)
    o = OS.resolve(S.render())
    err = rel_mse(g, o)
    assert err < 1e-3, err


def test_volume_config_band_at_its_own_size(gpu_ctx, scene_dir):
    """The heterogeneous-volume workload at its own size: 1024x1024, 64 spp, depth 32, a
    256^3 fBm density grid (sigma_t max 20, albedo 0.9, HG g 0.6) behind a transform
    medium and a 327,680-triangle displaced sphere with a GGX conductor. The whole frame
    renders through the wavefront (32 M-state queue, multi-bounce graphs, shadow streams);
    a band of rows through the sphere and the densest fog is compared with the oracle,
    which follows the same sampler and shadow-transmittance streams."""
    p = scenes.volume(out_dir=scene_dir / "volume-c2")
    sc = gpu_ctx.load_scene(p).build()
    info = sc.info()
    assert (info.width, info.height, info.spp, info.max_depth) == (1024, 1024, 64, 32)
    assert info.triangles >= 327680 and info.media >= 2
    stats = {}
    g = gpu_ctx.render(sc, stats=stats).astype(np.float64)
    assert stats["paths"] == 1024 * 1024 * 64 and stats["traversal_errors"] == 0
    assert np.isfinite(g).all()
    r0, r1 = 496, 528
    S = OS.Scene(p)
    o = OS.resolve(S.render(pixel_begin=r0 * 1024, pixel_end=r1 * 1024)[r0:r1])
    err = rel_mse(g[r0:r1], o)
    assert err < 1e-3, err
