"""G-buffer outputs and post-processing on the GPU.

  * albedo / normal g-buffers (wavefront/shade.cpp:133-139, 195-202 and the preview
    resolve, preview.cpp:27-78) against the oracle's first-hit g-buffer for the same
    sampler streams;
  * the ACES tone map kernel (postprocess/tonemap.cpp:14-53) against its formula;
  * a scene's post_processors list run by btrc_render (tonemap, then save of colour,
    albedo and normal), and the denoise entry (edge-avoiding a-trous filter standing in
    for the closed OptiX denoiser) against its NumPy restatement."""
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


@pytest.mark.parametrize("guides", [False, True])
def test_denoise_kernel_matches_oracle(gpu_ctx, guides):
    # HDR noise over piecewise-constant albedo / normal regions; the CUDA a-trous filter
    # against its NumPy restatement (FMA contraction and expf rounding: 1e-4 relative)
    import torch
    from oracle import denoise as OD
    rng = np.random.default_rng(31)
    h, w = 48, 64
    reg = (np.arange(w)[None, :] // 16 + 2 * (np.arange(h)[:, None] // 24)) % 4
    alb = rng.uniform(0.1, 0.9, (4, 3)).astype(np.float32)[reg]
    n = rng.normal(size=(4, 3))
    nrm = (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(np.float32)[reg]
    img = (3.0 * alb * rng.exponential(1.0, (h, w, 3))).astype(np.float32)
    d_img = torch.from_numpy(img).cuda()
    d_alb = torch.from_numpy(np.ascontiguousarray(alb)).cuda() if guides else None
    d_nrm = torch.from_numpy(np.ascontiguousarray(nrm)).cuda() if guides else None
    gpu_ctx.denoise_atrous(d_img, w, h, d_alb, d_nrm)
    torch.cuda.synchronize()
    got = d_img.cpu().numpy()
    want = OD.atrous(img, alb if guides else None, nrm if guides else None)
    assert np.allclose(got, want, rtol=1e-4, atol=1e-6), np.abs(got - want).max()
    # noise within each region falls; with the guides the regions keep their own colours
    within = lambda a: np.mean([a[reg == r].std(0).mean() for r in range(4)])
    assert within(got) < 0.5 * within(img)
    # an empty image is a no-op
    gpu_ctx.denoise_atrous(None, 0, 0)


def test_post_processors_denoise(gpu_ctx, tmp_path):
    # the scene's denoise entry runs the a-trous filter on the render, guided by the
    # renderer's albedo / normal g-buffers, and brings a 4-spp render closer to the
    # converged image
    from oracle import denoise as OD
    from tests.util import rel_mse
    p = scenes.cornell(out_dir=tmp_path, width=96, height=72, spp=4)
    scene = json.loads(p.read_text())
    scene["renderer"]["albedo"] = True
    scene["renderer"]["normal"] = True
    scene["post_processors"] = {"type": "denoise"}
    q = tmp_path / "denoise.json"
    q.write_text(json.dumps(scene))
    sc = gpu_ctx.load_scene(q).build()
    raw = gpu_ctx.render(sc)
    alb = np.zeros_like(raw)
    nrm = np.zeros_like(raw)
    out = gpu_ctx.render(sc, post_process=True, albedo=alb, normal=nrm)
    # raw comes from a second render of the same paths (film sums differ in atomic order)
    assert np.allclose(out, OD.atrous(raw, alb, nrm), rtol=1e-3, atol=1e-4)
    ref = gpu_ctx.render(sc, spp=1024)
    assert rel_mse(out, ref) < 0.5 * rel_mse(raw, ref)