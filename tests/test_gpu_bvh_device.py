"""Device BVH builder (PLOC clustering, the 8-wide collapse and node emission on the GPU).

It writes the host builder's node layout, so the host builder's structure checks apply
unchanged; traversal through a device-built tree must find exactly the oracle's hits
(closest hits do not depend on the tree); a render through it must equal the render
through the host-built tree."""
import json

import numpy as np
import pytest

import oracle
from btrc_gb300 import scenes
from oracle import scene as OS
from tests.test_bvh_structure import check_structure
from tests.test_gpu_trace import _gpu_trace
from tests.util import edge_rays

pytestmark = pytest.mark.gpu


def _duplicates_scene(out, copies=3000, seed=9):
    """Many identical triangles (equal boxes: every union area ties) plus a single
    triangle scene beside them, to exercise the clustering's tie rule."""
    out.mkdir(parents=True, exist_ok=True)
    rng = np.random.default_rng(seed)
    base = rng.uniform(-0.5, 0.5, (3, 3))
    v = np.concatenate([np.repeat(base[None], copies, 0), rng.uniform(-1, 1, (200, 3, 3))])
    scenes.write_obj(out / "dup.obj", v.reshape(-1, 3), np.arange(len(v) * 3).reshape(-1, 3))
    scene = {
        "width": 32, "height": 32,
        "camera": {"type": "pinhole", "eye": [0.0, 0.0, 4.0], "dst": [0.0, 0.0, 0.0], "up": [0.0, 1.0, 0.0],
                   "fov_y": {"deg": 50.0}},
        "renderer": {"type": "wfpt", "spp": 1},
        "scene": {"entities": [{"geometry": {"type": "triangle_mesh", "filename": "$env{scene_directory}/dup.obj"},
                                "material": {"type": "diffuse", "color": [0.5, 0.5, 0.5]}}]},
    }
    p = out / "scene.json"
    p.write_text(json.dumps(scene))
    return p


def _single_scene(out):
    out.mkdir(parents=True, exist_ok=True)
    v = np.array([[-1.0, -1.0, 0.0], [1.0, -1.0, 0.0], [0.0, 1.0, 0.0]])
    scenes.write_obj(out / "one.obj", v, np.arange(3).reshape(1, 3))
    scene = {
        "width": 16, "height": 16,
        "camera": {"type": "pinhole", "eye": [0.0, 0.0, 4.0], "dst": [0.0, 0.0, 0.0], "up": [0.0, 1.0, 0.0],
                   "fov_y": {"deg": 50.0}},
        "renderer": {"type": "wfpt", "spp": 1},
        "scene": {"entities": [{"geometry": {"type": "triangle_mesh", "filename": "$env{scene_directory}/one.obj"},
                                "material": {"type": "diffuse", "color": [0.5, 0.5, 0.5]}}]},
    }
    p = out / "scene.json"
    p.write_text(json.dumps(scene))
    return p


def _path(which, scene_dir):
    if which == "cornell":
        return scenes.cornell(out_dir=scene_dir / "cornell")
    if which == "soup":
        return scenes.random_soup(scene_dir / "soup", seed=5, n_tris=20000, n_instances=4)
    if which == "duplicates":
        return _duplicates_scene(scene_dir / "dup")
    if which == "single":
        return _single_scene(scene_dir / "single")
    return scenes.terrain(seed=7, width=64, height=64, spp=1, grid=128, instances=8, out_dir=scene_dir / "terrain")


@pytest.mark.parametrize("which", ["cornell", "soup", "duplicates", "single", "terrain"])
def test_device_bvh_structure(gpu_ctx, scene_dir, which):
    sc = gpu_ctx.load_scene(_path(which, scene_dir)).build(builder="device")
    info = sc.info()
    assert info.bvh_builder == 1
    assert info.bvh_depth <= 32
    check_structure(sc)
    if which == "terrain":
        # the collapse keeps the nodes about as full as on host-built trees
        nodes, _ = sc.export_bvh()
        assert (nodes[:, 24:32] != 0).sum(1).mean() > 5.0


@pytest.mark.parametrize("which", ["soup", "duplicates", "terrain"])
def test_device_bvh_traversal_bitexact(gpu_ctx, scene_dir, which):
    path = _path(which, scene_dir)
    S = OS.Scene(path)
    rng = np.random.default_rng(3)
    n = 20000
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(-2, 2, (n, 3))
    rays[:, 4:7] = rng.normal(size=(n, 3))
    rays[:, 7] = 3.0e38
    seg = rng.random(n) < 0.3
    rays[seg, 7] = 1.0
    rays = np.concatenate([rays, edge_rays(rng, S.tris, 10000)])
    dev = gpu_ctx.load_scene(path).build(builder="device")
    host = gpu_ctx.load_scene(path).build(builder="host")
    d_flags, d_hits, d_occ = _gpu_trace(gpu_ctx, dev, rays)
    h_flags, h_hits, h_occ = _gpu_trace(gpu_ctx, host, rays)
    bvh = oracle.OracleBvh(S.tris, S.ids)
    o_flags, o_hits = bvh.closest(rays)
    o_occ = bvh.any(rays)
    bad = np.nonzero(d_flags != o_flags)[0]
    assert len(bad) == 0, f"{len(bad)} flag mismatches, first {bad[:5]}"
    hit = o_flags != 0
    assert np.array_equal(d_hits[hit].view(np.uint32), o_hits[hit].view(np.uint32))
    assert np.array_equal(d_occ, o_occ)
    assert np.array_equal(d_flags, h_flags) and np.array_equal(d_occ, h_occ)
    assert hit.mean() > 0.05


def test_device_bvh_render_equals_host_build(gpu_ctx, scene_dir):
    path = scenes.terrain(seed=7, width=64, height=64, spp=4, grid=128, instances=8, out_dir=scene_dir / "terrain-r")
    dev = gpu_ctx.load_scene(path).build(builder="device")
    host = gpu_ctx.load_scene(path).build(builder="host")
    a = gpu_ctx.render(dev)
    b = gpu_ctx.render(host)
    # the same paths hit the same triangles; only the film's atomic accumulation order
    # may differ
    assert np.allclose(a, b, rtol=1e-5, atol=1e-6)


def test_device_bvh_batch_build(gpu_ctx, scene_dir):
    paths = [scenes.random_soup(scene_dir / f"bsoup{k}", seed=20 + k, n_tris=3000 + 1000 * k, n_instances=2)
             for k in range(6)]
    built = gpu_ctx.load_build_scenes([str(p) for p in paths], builder="device")
    for p, sc in zip(paths, built):
        assert sc.info().bvh_builder == 1
        check_structure(sc)


def test_device_bvh_is_deterministic(gpu_ctx, scene_dir):
    """Merges claim node slots with atomics, so binary node numbers vary from run to run;
    the emitted wide tree depends only on the tree's shape and must not."""
    path = _path("soup", scene_dir)
    a = gpu_ctx.load_scene(path).build(builder="device")
    b = gpu_ctx.load_scene(path).build(builder="device")
    na, ta = a.export_bvh()
    nb, tb = b.export_bvh()
    assert np.array_equal(na, nb) and np.array_equal(ta, tb)
