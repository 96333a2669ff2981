"""G-buffer outputs and post-processing on the GPU.

  * albedo / normal g-buffers (wavefront/shade.cpp:133-139, 195-202 and the preview
    resolve, preview.cpp:27-78) against the oracle's first-hit g-buffer for the same
    sampler streams;
  * the ACES tone map kernel (postprocess/tonemap.cpp:14-53) against its formula;
  * a scene's post_processors list run by btrc_render (tonemap, then save of colour,
    albedo and normal), and a denoise entry reported as unsupported."""
import json

import numpy as np
import pytest

import btrc_gb300 as B
from btrc_gb300 import scenes
from oracle import scene as OS
from tests.test_image_io import read_exr, read_png

pytestmark = pytest.mark.gpu


def aces(x):
    x = x.astype(np.float32)
    v = (x * (np.float32(2.51) * x + np.float32(0.03))) / (x * (np.float32(2.43) * x + np.float32(0.59)) +
                                                           np.float32(0.14))
    return np.clip(v, 0, 1)


@pytest.mark.parametrize("variant", ["diffuse", "glass", "textured"])
def test_gbuffer_matches_oracle(gpu_ctx, scene_dir, variant):
    if variant == "textured":
        # albedo from image textures, normals from normal maps
        p = scenes.textured(out_dir=scene_dir / "textured", width=48, height=48, spp=16)
    else:
        p = scenes.cornell(out_dir=scene_dir / "cornell", width=48, height=48, spp=16, variant=variant)
    sc = gpu_ctx.load_scene(p).build()
    alb = np.zeros((48, 48, 3), np.float32)
    nrm = np.zeros((48, 48, 3), np.float32)
    gpu_ctx.render(sc, albedo=alb, normal=nrm)
    S = OS.Scene(p)
    film, aov = S.render_aov()
    oa, on = OS.resolve_aov(film, aov)
    # first hits coincide except where a camera ray grazes a silhouette
    da = np.abs(alb - oa).max(-1)
    dn = np.abs(nrm - on).max(-1)
    assert (da < 1e-4).mean() > 0.97 and da.mean() < 2e-3, (da.mean(), (da < 1e-4).mean())
    assert (dn < 1e-4).mean() > 0.97 and dn.mean() < 5e-3, (dn.mean(), (dn < 1e-4).mean())
    assert np.allclose(np.linalg.norm(nrm, axis=-1)[np.linalg.norm(on, axis=-1) > 0], 1, atol=1e-5)


def test_tonemap_kernel(gpu_ctx):
    import torch
    rng = np.random.default_rng(7)
    for ch in (3, 4):
        x = rng.uniform(0, 8, (33, 17, ch)).astype(np.float32)
        d = torch.from_numpy(x).cuda()
        gpu_ctx.tonemap_aces(d, 17, 33, ch, exposure=0.7)
        torch.cuda.synchronize()
        got = d.cpu().numpy()
        want = aces(x[..., :3] * np.float32(0.7))
        assert np.allclose(got[..., :3], want, rtol=2e-6, atol=1e-7)
        if ch == 4:
            assert np.array_equal(got[..., 3], x[..., 3])


def _post_scene(tmp_path, post):
    p = scenes.cornell(out_dir=tmp_path, width=40, height=30, spp=8)
    scene = json.loads(p.read_text())
    scene["renderer"]["albedo"] = True
    scene["renderer"]["normal"] = True
    scene["post_processors"] = post
    q = tmp_path / "post.json"
    q.write_text(json.dumps(scene))
    return q


def test_post_processors_tonemap_then_save(gpu_ctx, tmp_path):
    post = [{"type": "tonemap", "exposure": 1.5},
            {"type": "save", "gamma": 2.2, "color": "$env{scene_directory}/color.png",
             "albedo": "$env{scene_directory}/albedo.exr", "normal": "$env{scene_directory}/normal.exr"}]
    p = _post_scene(tmp_path, post)
    sc = gpu_ctx.load_scene(p).build()
    raw = gpu_ctx.render(sc)
    alb = np.zeros_like(raw)
    out = gpu_ctx.render(sc, post_process=True, albedo=alb)
    # the returned image is the tone-mapped render
    assert np.allclose(out, aces(raw * np.float32(1.5)), rtol=1e-4, atol=1e-5)
    png = read_png(tmp_path / "color.png").astype(np.int64)
    want = np.minimum((np.power(out, np.float32(1 / 2.2)) * 256).astype(np.int64), 255)
    assert np.abs(png[..., :3] - want).max() <= 1 and (png[..., 3] == 255).all()
    ex = read_exr(tmp_path / "albedo.exr")
    assert np.array_equal(np.stack([ex["R"], ex["G"], ex["B"]], -1), alb)
    nx = read_exr(tmp_path / "normal.exr")
    n = np.stack([nx["R"], nx["G"], nx["B"]], -1)
    assert np.allclose(np.linalg.norm(n, axis=-1), 1, atol=1e-5)


def test_post_processors_denoise_unsupported(gpu_ctx, tmp_path):
    p = _post_scene(tmp_path, {"type": "denoise"})
    sc = gpu_ctx.load_scene(p).build()
    gpu_ctx.render(sc)  # without post-processing the scene renders
    with pytest.raises(B.BtrcError) as e:
        gpu_ctx.render(sc, post_process=True)
    assert e.value.status == 8
