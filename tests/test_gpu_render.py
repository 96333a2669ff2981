"""Whole-image parity: the GPU wavefront renderer against the oracle renderer on the same
scene JSON. Both use the same per-pixel sampler streams, so their paths coincide except
where FP32 transcendental rounding flips a branch; the images must agree far inside the
noise (relMSE bound below) and the per-pixel difference must be consistent with zero
mean (no bias)."""
import numpy as np
import pytest

from btrc_gb300 import scenes
from oracle import scene as OS
from tests.util import rel_mse

pytestmark = pytest.mark.gpu


def _render_both(ctx, path, spp, batches=4):
    sc = ctx.load_scene(path).build()
    stats = {}
    g = ctx.render(sc, spp=spp, stats=stats)
    S = OS.Scene(path)
    per = spp // batches
    films = [S.render(spp=per, sample_begin=k * per) for k in range(batches)]
    imgs = np.stack([OS.resolve(f) for f in films])
    o = imgs.mean(0)
    var = imgs.var(0, ddof=1) / batches
    return g.astype(np.float64), o, var, stats


def test_cornell_halton_gaussian(gpu_ctx, scene_dir):
    p = scenes.cornell(out_dir=scene_dir / "cornell", width=64, height=64, spp=256)
    g, o, var, stats = _render_both(gpu_ctx, p, 256)
    assert stats["paths"] == 64 * 64 * 256
    assert stats["traversal_errors"] == 0
    assert np.isfinite(g).all()
    err = rel_mse(g, o)
    assert err < 1e-3, err
    z = np.mean((g - o) ** 2 / (2 * var + 1e-8))
    assert z < 2.0, z


def test_cornell_glass_and_mirror(gpu_ctx, scene_dir):
    # delta dielectric (Fresnel-chosen reflection / refraction with the eta^2 radiance
    # factor) and a Schlick-tinted mirror; caustics through the glass make this the
    # noisiest scene, hence more spp
    # (4096 spp, the image bar's sample count: a path that rounding sends the other way
    # through the glass weighs 1 / spp)
    p = scenes.cornell(out_dir=scene_dir / "cornell", width=48, height=48, spp=4096, variant="glass")
    g, o, var, stats = _render_both(gpu_ctx, p, 4096, batches=8)
    assert stats["traversal_errors"] == 0
    assert np.isfinite(g).all()
    err = rel_mse(g, o)
    assert err < 1e-3, err
    z = np.mean((g - o) ** 2 / (2 * var + 1e-8))
    assert z < 2.0, z


def test_textured_ibl_scene(gpu_ctx, scene_dir):
    # PNG image textures (sRGB, wrap / mirror / border addressing, point and linear
    # filters), texture expressions (mul, add, uv transform), normal maps and an HDR
    # environment light with its tile importance table
    p = scenes.textured(out_dir=scene_dir / "textured", width=64, height=48, spp=2048)
    g, o, var, stats = _render_both(gpu_ctx, p, 2048, batches=8)
    assert stats["traversal_errors"] == 0
    assert np.isfinite(g).all()
    err = rel_mse(g, o)
    assert err < 1e-3, err
    z = np.mean((g - o) ** 2 / (2 * var + 1e-8))
    assert z < 2.0, z


def test_terrain_disney_sky(gpu_ctx, scene_dir):
    p = scenes.terrain(out_dir=scene_dir / "terrain-small", width=96, height=54, spp=128, grid=96, instances=24)
    g, o, var, stats = _render_both(gpu_ctx, p, 128)
    assert stats["traversal_errors"] == 0
    err = rel_mse(g, o)
    assert err < 1e-3, err
    z = np.mean((g - o) ** 2 / (2 * var + 1e-8))
    assert z < 2.0, z


def test_render_reuses_context_and_cancel_flag_resets(gpu_ctx, scene_dir):
    p = scenes.cornell(out_dir=scene_dir / "cornell", width=32, height=32, spp=4)
    sc = gpu_ctx.load_scene(p).build()
    a = gpu_ctx.render(sc)
    b = gpu_ctx.render(sc)
    # deterministic: same sampler streams, same queue order -> same image up to atomic order
    assert np.allclose(a, b, rtol=1e-4, atol=1e-5)


def test_procedural_geometry_scene(gpu_ctx, tmp_path):
    # inline sphere / quad / box creators (smooth normals, texture coordinates, flat boxes)
    from tests.test_abi_loader import _procedural_scene
    p = _procedural_scene(tmp_path)
    g, o, var, stats = _render_both(gpu_ctx, p, 256)
    assert stats["traversal_errors"] == 0
    err = rel_mse(g, o)
    assert err < 1e-3, err


def test_tile_generation_matches_uniform(gpu_ctx, scene_dir):
    # renderer.tile (W/generate.cpp:56-60) orders the (pixel, sample) pairs pixel-major
    # instead of sample-major; every pair keeps its own sampler stream, so the two modes
    # trace the same paths and the images differ only by the order of the film atomics.
    # The state queue is smaller than the frame so that both orders need several refills.
    import json
    p = scenes.cornell(out_dir=scene_dir / "cornell", width=40, height=40, spp=64)
    scene = json.loads(p.read_text())
    scene["renderer"]["state_count"] = 8192
    uni = p.parent / "tile-off.json"
    uni.write_text(json.dumps(scene))
    scene["renderer"]["tile"] = True
    til = p.parent / "tile-on.json"
    til.write_text(json.dumps(scene))
    imgs = []
    for q in (uni, til):
        sc = gpu_ctx.load_scene(q).build()
        stats = {}
        imgs.append(gpu_ctx.render(sc, stats=stats).astype(np.float64))
        assert stats["paths"] == 40 * 40 * 64 and stats["traversal_errors"] == 0
        sc.close()
    a, b = imgs
    assert np.isfinite(a).all() and np.isfinite(b).all()
    assert np.allclose(a, b, rtol=1e-4, atol=1e-6), np.abs(a - b).max()


def test_scene_without_geometry_sees_the_sky(gpu_ctx, tmp_path):
    # no entities: an empty BVH, every camera ray misses and collects the gradient sky
    # (B/light/gradient_sky.cpp:20-40) at its direction, so the image is the oracle's
    # exactly up to the filter's weights
    import json
    scene = {"width": 32, "height": 24,
             "camera": {"type": "pinhole", "eye": [0, 0, 0], "dst": [0, 0.3, -1], "up": [0, 1, 0],
                        "fov_y": {"deg": 60}},
             "renderer": {"type": "wfpt", "spp": 16, "sampler": "independent"},
             "scene": {"entities": [],
                       "envir_light": {"type": "gradient_sky", "lower": [0.1, 0.2, 0.3], "upper": [0.9, 0.8, 0.5],
                                       "up": [0, 1, 0]}}}
    p = tmp_path / "sky.json"
    p.write_text(json.dumps(scene))
    g, o, var, stats = _render_both(gpu_ctx, p, 16)
    assert stats["traversal_errors"] == 0 and stats["paths"] == 32 * 24 * 16
    assert stats["extension_rays"] == 32 * 24 * 16  # one per path, all misses
    assert np.isfinite(g).all()
    assert np.allclose(g, o, rtol=1e-4, atol=1e-5), np.abs(g - o).max()
    # the sky brightens upwards: top rows brighter than bottom rows in red
    assert g[0, :, 0].mean() > g[-1, :, 0].mean()
