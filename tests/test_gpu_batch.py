"""Batched rendering of uneven scenes (btrc_render_batch): every scene rendered through
the concurrent lanes, with autotuned queue capacity and grid size, gives the image the
single-scene renderer gives (same sampler streams; only the order of film atomics
differs), and the per-scene statistics account for every path."""
import numpy as np
import pytest

from btrc_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_batch_matches_single_renders(gpu_ctx, scene_dir):
    paths = scenes.batch(count=6, seed=77, out_dir=scene_dir / "batch")
    scs = [gpu_ctx.load_scene(p).build() for p in paths]
    infos = [s.info() for s in scs]
    outs = [np.zeros((i.height, i.width, 3), np.float32) for i in infos]
    stats, total = gpu_ctx.render_batch(scs, outs, lanes=3, autotune=True)
    assert total > 0
    for s, o, st, i in zip(scs, outs, stats, infos):
        ref = gpu_ctx.render(s)
        assert st["paths"] == i.width * i.height * i.spp
        assert 0 <= st["lane"] < 3 and st["capacity"] > 0 and st["grid_pct"] in (50, 100)
        assert 0 < st["ms"] <= st["done_ms"] <= total * 1.001
        assert np.allclose(o, ref, rtol=1e-4, atol=1e-5)
    # within a lane, scenes complete in the order they were rendered
    for lane in range(3):
        done = [st["done_ms"] for st in stats if st["lane"] == lane]
        assert len(done) <= 1 or np.all(np.diff(sorted(done)) > 0)
    # device outputs, no autotune, one lane
    import torch
    outs_d = [torch.zeros((i.height, i.width, 3), dtype=torch.float32, device="cuda") for i in infos]
    gpu_ctx.render_batch(scs, outs_d, lanes=1, autotune=False)
    torch.cuda.synchronize()
    for o, h in zip(outs_d, outs):
        assert np.allclose(o.cpu().numpy(), h, rtol=1e-4, atol=1e-5)
    for s in scs:
        s.close()


def test_merged_batch_matches_single_renders(gpu_ctx, scene_dir):
    """One merged pass (every scene's paths in one queue, one set of stage kernels, each
    path's scene read from its film row) gives every scene the image of its own render:
    same sampler streams, rebased BVH / instance / light indices, per-scene cameras,
    lights, sky and path-length rules."""
    import torch
    paths = scenes.batch(count=6, seed=78, out_dir=scene_dir / "batch-merged")
    scs = [gpu_ctx.load_scene(p).build() for p in paths]
    infos = [s.info() for s in scs]
    refs = [gpu_ctx.render(s) for s in scs]
    outs = [np.zeros((i.height, i.width, 3), np.float32) for i in infos]
    stats, total = gpu_ctx.render_batch(scs, outs, autotune=False, merged=True)
    assert total > 0
    for o, r, st, i in zip(outs, refs, stats, infos):
        assert st["paths"] == i.width * i.height * i.spp
        assert 0 < st["ms"] <= total and st["done_ms"] == st["ms"]
        assert np.allclose(o, r, rtol=1e-4, atol=1e-5), np.abs(o - r).max()
    # the queue census: a scene is complete no later than the pass, and the scene with the
    # fewest paths (queued first) no later than the one with the most
    few = min(range(len(stats)), key=lambda k: stats[k]["paths"])
    most = max(range(len(stats)), key=lambda k: stats[k]["paths"])
    assert stats[few]["done_ms"] <= stats[most]["done_ms"]
    # autotuned, device outputs; the concatenated scene is reused
    outs_d = [torch.zeros((i.height, i.width, 3), dtype=torch.float32, device="cuda") for i in infos]
    stats, _ = gpu_ctx.render_batch(scs, outs_d, autotune=True, merged=True)
    torch.cuda.synchronize()
    for o, r, st in zip(outs_d, refs, stats):
        assert st["block"] in (128, 256) and st["grid_pct"] in (50, 100) and st["capacity"] > 0
        assert np.allclose(o.cpu().numpy(), r, rtol=1e-4, atol=1e-5)
    for s in scs:
        s.close()


def test_merged_batch_refuses_media(gpu_ctx, scene_dir):
    import btrc_gb300 as B
    p = scenes.cornell(out_dir=scene_dir / "cornell", width=48, height=48, spp=4, variant="fog")
    sc = gpu_ctx.load_scene(p).build()
    out = np.zeros((48, 48, 3), np.float32)
    with pytest.raises(B.BtrcError) as e:
        gpu_ctx.render_batch([sc], [out], merged=True)
    assert e.value.status == 8
    sc.close()


def test_batches_of_device_built_and_two_level_scenes(gpu_ctx, scene_dir):
    """Device-built BVHs go through the merged pass and two-level scenes through the lanes,
    each giving the image of the scene's own render."""
    paths = scenes.batch(count=4, seed=79, out_dir=scene_dir / "batch-forms")
    dev = gpu_ctx.load_build_scenes([str(p) for p in paths], builder="device")
    infos = [s.info() for s in dev]
    assert all(i.bvh_builder == 1 for i in infos)
    refs = [gpu_ctx.render(s) for s in dev]
    outs = [np.zeros((i.height, i.width, 3), np.float32) for i in infos]
    gpu_ctx.render_batch(dev, outs, autotune=False, merged=True)
    for o, r in zip(outs, refs):
        assert np.allclose(o, r, rtol=1e-4, atol=1e-5)
    two = gpu_ctx.load_build_scenes([str(p) for p in paths], two_level=True)
    assert all(s.info().two_level == 1 for s in two)
    refs2 = [gpu_ctx.render(s) for s in two]
    outs2 = [np.zeros((i.height, i.width, 3), np.float32) for i in infos]
    gpu_ctx.render_batch(two, outs2, lanes=2, autotune=False)
    for o, r in zip(outs2, refs2):
        assert np.allclose(o, r, rtol=1e-4, atol=1e-5)
    for s in dev + two:
        s.close()
