"""Neural radiance cache on the GPU against the NumPy oracle (oracle/nrc.py).

  * forward: the fused tensor-core MLP's predictions equal the oracle's BF16 forward;
  * gradients: the loss, the weight gradients of every layer and the hash-feature
    gradients of one training step match the oracle (BF16 rounding points restated, so
    only accumulation order differs);
  * learning: Adam on fresh batches of a smooth synthetic radiance field lowers the loss
    by an order of magnitude."""
import numpy as np
import pytest

import btrc_gb300 as B
from oracle import nrc as ON

pytestmark = pytest.mark.gpu

LO, HI = [-1.0, -0.5, -2.0], [1.0, 1.5, 0.0]


def _samples(rng, n, field=None):
    s = np.zeros((n, 16), np.float32)
    s[:, 0:3] = rng.uniform(LO, HI, (n, 3))
    d = rng.normal(size=(n, 3)); s[:, 3:6] = d / np.linalg.norm(d, axis=1, keepdims=True)
    nn = rng.normal(size=(n, 3)); s[:, 6:9] = nn / np.linalg.norm(nn, axis=1, keepdims=True)
    s[:, 9] = rng.uniform(0, 1, n)
    s[:, 10:13] = rng.uniform(0, 1, (n, 3))
    s[:, 13:16] = rng.uniform(0, 2, (n, 3)) if field is None else field(s)
    return s


def _cache(gpu_ctx, seed=3, hash_scale=0.5):
    c = B.RadianceCache(gpu_ctx, LO, HI, seed=seed)
    rng = np.random.default_rng(seed)
    h = rng.uniform(-hash_scale, hash_scale, B.NRC_HASH_FLOATS).astype(np.float32)
    c.set_params(1, h)
    return c, h


def test_forward_matches_oracle(gpu_ctx):
    import torch
    c, h = _cache(gpu_ctx)
    w = c.params(0)
    s = _samples(np.random.default_rng(1), 1000)
    q = torch.from_numpy(np.ascontiguousarray(s[:, :13])).cuda()
    out = torch.zeros((1000, 4), dtype=torch.float32, device="cuda")
    c.infer(q, 1000, out)
    torch.cuda.synchronize()
    g = out.cpu().numpy()[:, :3]
    x0, _ = ON.encode(s[:, :13], h, LO, HI)
    _, y = ON.forward(x0, w)
    err = np.abs(g - y[:, :3])
    assert err.max() < 2e-2 * (np.abs(y[:, :3]).max() + 1e-3), err.max()
    assert np.mean(err) < 2e-3 * (np.abs(y[:, :3]).mean() + 1e-3), np.mean(err)
    c.close()


def test_gradients_match_oracle(gpu_ctx):
    import torch
    c, h = _cache(gpu_ctx, seed=5)
    w = c.params(0)
    s = _samples(np.random.default_rng(2), 777)
    d = torch.from_numpy(s).cuda()
    loss = c.train(d, len(s), apply_adam=False)
    gw, gh = c.params(2), c.params(3)
    oloss, ow, oh, _ = ON.loss_and_grads(s, w, h, LO, HI)
    assert abs(loss - oloss) < 1e-3 * abs(oloss) + 1e-6, (loss, oloss)
    o = 0
    for l, (k, n) in enumerate(ON.layer_shapes()):
        a, b = gw[o:o + k * n], ow[o:o + k * n]
        o += k * n
        rel = np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30)
        assert rel < 2e-2, (l, rel)
        assert np.dot(a, b) / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30) > 0.999, l
    touched = oh != 0
    rel = np.linalg.norm(gh[touched] - oh[touched]) / np.linalg.norm(oh[touched])
    assert rel < 2e-2, rel
    assert np.all(gh[~touched] == 0)
    c.close()


def test_training_reduces_loss(gpu_ctx):
    import torch
    c = B.RadianceCache(gpu_ctx, LO, HI, seed=7)

    def field(s):
        x, y, z = s[:, 0], s[:, 1], s[:, 2]
        base = 0.6 + 0.4 * np.sin(3 * x) * np.cos(2 * y) + 0.2 * z
        return (base[:, None] * (0.3 + s[:, 10:13]) * (0.5 + 0.5 * s[:, 8:9] ** 2)).astype(np.float32)
    rng = np.random.default_rng(9)
    losses = []
    for step in range(300):
        s = _samples(rng, 1 << 14, field)
        losses.append(c.train(torch.from_numpy(s).cuda(), len(s)))
    first, last = np.mean(losses[:10]), np.mean(losses[-10:])
    assert np.isfinite(losses).all()
    assert last < first / 10, (first, last)
    c.close()


def _relmse(a, r):
    return float(np.mean((a - r) ** 2 / (r ** 2 + 1e-2)))


def test_cache_render_off_matches_plain_and_training_helps(gpu_ctx, scene_dir):
    # with the cache off a frame is exactly the plain renderer's single sample; with it on,
    # the trained cache must beat terminating paths into the untrained network (the
    # method without learning) by a wide margin on the same frames
    from btrc_gb300 import scenes
    p = scenes.cornell(out_dir=scene_dir / "cornell", width=64, height=64, spp=1)
    sc = gpu_ctx.load_scene(p).build()
    info = sc.info()
    ref = gpu_ctx.render(sc, spp=2048).astype(np.float64)
    cache = B.RadianceCache(gpu_ctx, info.world_min, info.world_max, seed=1)
    f0 = cache.render_frame(sc, 0, terminate_vertex=-1, train_stride=0, train_steps=0)
    assert np.array_equal(f0, gpu_ctx.render(sc, spp=1))
    frames = 96
    res = {}
    for mode, steps in (("trained", 4), ("untrained", 0)):
        c = B.RadianceCache(gpu_ctx, info.world_min, info.world_max, seed=2)
        acc = np.zeros_like(ref)
        st, losses = {}, []
        for f in range(frames):
            acc += c.render_frame(sc, f, terminate_vertex=1, train_stride=4, train_steps=steps, train_batch=4096,
                                  stats=st)
            losses.append(st["loss"])
        assert st["queries"] > 0.5 * 64 * 64
        res[mode] = _relmse(acc / frames, ref)
        if steps:
            assert st["train_samples"] > 0 and np.isfinite(losses).all()
            assert np.mean(losses[-8:]) < np.mean(losses[:4])
        c.close()
    assert res["trained"] < 0.5 * res["untrained"], res


def test_path_spread_termination(gpu_ctx, scene_dir):
    """The path-spread rule (Mueller et al. 2021, section 4): with a vanishing threshold a
    path ends at its first non-delta vertex after one bounce, as with the depth rule; with
    a huge one no path ever reaches the cache; in between fewer paths end there."""
    from btrc_gb300 import scenes
    p = scenes.cornell(out_dir=scene_dir / "cornell", width=64, height=64, spp=1)
    sc = gpu_ctx.load_scene(p).build()
    info = sc.info()
    c = B.RadianceCache(gpu_ctx, info.world_min, info.world_max, seed=2)
    counts = {}
    for name, kw in (("depth", {}), ("tiny", {"spread_threshold": 1e-12}), ("mid", {"spread_threshold": 1.0}),
                     ("huge", {"spread_threshold": 1e12})):
        st = {}
        img = c.render_frame(sc, 0, train_stride=0, train_steps=0, stats=st, **kw)
        assert np.isfinite(img).all()
        counts[name] = st["queries"]
    assert counts["huge"] == 0
    assert counts["depth"] > 0 and counts["tiny"] >= 0.95 * counts["depth"], counts
    assert counts["mid"] <= counts["tiny"], counts
    c.close()
    sc.close()
