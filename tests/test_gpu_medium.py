"""Participating media on the GPU.

  * ratio-tracking transmittance (builtin/btrc/builtin/medium/hetergeneous.cpp:75-106) is
    an unbiased estimator: its mean over many seeds must match exp(-sigma * L) for a
    constant-density grid behind a transform medium, within 4 standard errors, and
    exp(-integral of sigma) for a grid linear in x, y and z;
  * a homogeneous medium's Tr is the reference's closed form exp(-L sigma_t (1 - albedo));
  * a small heterogeneous-volume scene (text-format 32^3 grid, HG g = 0.6, GGX sphere)
    renders like the oracle (relMSE below 1e-3 and a bias z-test): shadow-ray
    transmittance draws from a stream seeded by the path's own sampler state on both
    sides, so the paths coincide as in the surface-only scenes;
  * volume primitives (`volumes[]`, core/btrc/core/volume.cpp:112-197): per-segment
    transmittance equals the oracle's when both draw the same PCG stream, and a Cornell box
    with three overlapping volumes (constant, grid and RGB-grid albedo) renders like the
    oracle."""
import json

import numpy as np
import pytest

from btrc_gb300 import scenes
from oracle import scene as OS
from tests.util import rel_mse, ramp_medium_scene, ramp_segments, ramp_tr_exact

pytestmark = pytest.mark.gpu


def _medium_scene(tmp, medium):
    cv, cf = scenes.box_inward((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5))
    scenes.write_obj(tmp / "cube.obj", cv, scenes.flip(cf))
    scene = {"width": 8, "height": 8,
             "camera": {"type": "pinhole", "eye": [0, 0, 3], "dst": [0, 0, 0], "up": [0, 1, 0], "fov_y": {"deg": 30}},
             "renderer": {"type": "wfpt", "spp": 1},
             "scene": {"entities": [{"geometry": {"type": "triangle_mesh", "filename": "$env{scene_directory}/cube.obj"},
                                     "material": {"type": "invisible"}, "inner_medium": medium}]}}
    p = tmp / "medium.json"
    p.write_text(json.dumps(scene))
    return p


def _tr(ctx, path, segs, seeds, medium_id=0):
    import torch
    sc = ctx.load_scene(path).build()
    n = len(segs)
    out = torch.zeros(n, dtype=torch.float32, device="cuda")
    ctx.medium_tr_batch(sc, medium_id, torch.from_numpy(segs.astype(np.float32)).cuda(),
                        torch.from_numpy(seeds.view(np.int64)).cuda(), n, out)
    torch.cuda.synchronize()
    return out.cpu().numpy().astype(np.float64)


def test_ratio_tracking_constant_grid(gpu_ctx, tmp_path):
    sigma = 3.0
    grid = np.full((4, 4, 4), sigma, np.float32)
    scenes.write_grid_text(tmp_path / "g.txt", grid)
    medium = {"type": "transform", "world_to_local": {"scale": [2, 2, 2]},
              "medium": {"type": "hetergeneous", "sigma_t": {"type": "array", "text": "$env{scene_directory}/g.txt"},
                         "albedo": 0.8, "g": 0.0}}
    p = _medium_scene(tmp_path, medium)
    n = 200000
    for L in (0.1, 0.4, 0.9):
        segs = np.tile([[-0.45, 0.0, 0.0, -0.45 + L, 0.0, 0.0]], (n, 1))
        tr = _tr(gpu_ctx, p, segs, np.arange(n, dtype=np.uint64) * 7919 + 17)
        want = np.exp(-sigma * L)
        se = tr.std() / np.sqrt(n)
        assert abs(tr.mean() - want) < 4 * se + 1e-6, (L, tr.mean(), want, se)
        # sigma_max == sigma: every tentative collision is real, so each estimate is 0 or 1
        # up to the rounding of the interpolated density
        assert np.all(np.minimum(np.abs(tr), np.abs(tr - 1.0)) < 1e-6)


def test_ratio_tracking_linear_grid(gpu_ctx, tmp_path):
    """Density linear in x, y and z (trilinear filtering reproduces it exactly): the mean
    ratio-tracking estimate along each segment equals exp(-length * sigma(midpoint))."""
    p = ramp_medium_scene(tmp_path)
    n = 200000
    for s in ramp_segments():
        segs = np.tile(s, (n, 1))
        tr = _tr(gpu_ctx, p, segs, np.arange(n, dtype=np.uint64) * 7919 + 3)
        want = float(ramp_tr_exact(s.astype(np.float32).astype(np.float64)))
        se = tr.std() / np.sqrt(n)
        assert abs(tr.mean() - want) < 4.5 * se, (s, tr.mean(), want, se)


def test_homogeneous_closed_form(gpu_ctx, tmp_path):
    medium = {"type": "homogeneous", "sigma_t": 2.5, "albedo": [0.2, 0.5, 0.9]}
    p = _medium_scene(tmp_path, medium)
    segs = np.array([[0, 0, 0, 0.3, 0, 0], [0, 0, 0, 0, 0, 0.7]], np.float32)
    tr = _tr(gpu_ctx, p, segs, np.array([1, 2], np.uint64))
    # the batch hook returns the red channel
    want = np.exp(-np.array([0.3, 0.7]) * 2.5 * (1 - 0.2))
    assert np.allclose(tr, want, rtol=1e-5)


def test_volume_scene_matches_oracle(gpu_ctx, scene_dir):
    p = scenes.volume(out_dir=scene_dir / "volume-small", width=48, height=48, spp=256, grid_res=32,
                      sphere_level=4, text_grid=True)
    sc = gpu_ctx.load_scene(p).build()
    stats = {}
    g = gpu_ctx.render(sc, stats=stats).astype(np.float64)
    assert stats["traversal_errors"] == 0 and np.isfinite(g).all()
    S = OS.Scene(p)
    batches = 8
    per = 256 // batches
    imgs = np.stack([OS.resolve(S.render(spp=per, sample_begin=k * per)) for k in range(batches)])
    o = imgs.mean(0)
    var = imgs.var(0, ddof=1) / batches
    # both sides follow the same sampler streams, and each shadow ray's transmittance
    # stream is seeded from its path's sampler state, so paths coincide up to rounding
    z = np.mean((g - o) ** 2 / (2 * var + 1e-8))
    assert z < 2.0, z
    assert rel_mse(g, o) < 1e-3


def test_volume_primitives_tr_matches_oracle(gpu_ctx, scene_dir):
    p = scenes.cornell(out_dir=scene_dir / "cornell", width=48, height=48, spp=256, variant="fog")
    S = OS.Scene(p)
    rng = np.random.default_rng(5)
    n = 20000
    lo, hi = np.array([-0.5, -0.5, 0.1]), np.array([0.5, 0.5, 1.1])
    segs = np.concatenate([rng.uniform(lo, hi, (n, 3)), rng.uniform(lo, hi, (n, 3))], 1).astype(np.float32)
    seeds = rng.integers(0, 2 ** 62, n, dtype=np.uint64)
    g = _tr(gpu_ctx, p, segs, seeds, medium_id=S.vacuum)
    o = S.medium_tr(S.vacuum, segs, seeds).astype(np.float64)
    assert np.isfinite(g).all()
    # same random numbers on both sides: equal up to rounding, except where rounding moves a
    # tentative collision across a segment end
    close = np.abs(g - o) <= 1e-4 + 1e-4 * np.abs(o)
    assert close.mean() > 0.995, close.mean()
    assert (o < 1).mean() > 0.3  # most segments cross some volume
    assert abs(g.mean() - o.mean()) < 3e-3


def test_volume_primitives_scene_matches_oracle(gpu_ctx, scene_dir):
    p = scenes.cornell(out_dir=scene_dir / "cornell", width=48, height=48, spp=256, variant="fog")
    sc = gpu_ctx.load_scene(p).build()
    stats = {}
    g = gpu_ctx.render(sc, stats=stats).astype(np.float64)
    assert stats["traversal_errors"] == 0 and np.isfinite(g).all()
    S = OS.Scene(p)
    batches = 8
    per = 256 // batches
    imgs = np.stack([OS.resolve(S.render(spp=per, sample_begin=k * per)) for k in range(batches)])
    o = imgs.mean(0)
    var = imgs.var(0, ddof=1) / batches
    z = np.mean((g - o) ** 2 / (2 * var + 1e-8))
    assert z < 2.0, z
    assert rel_mse(g, o) < 1e-3
