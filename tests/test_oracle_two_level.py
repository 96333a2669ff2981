"""CPU checks of the oracle's two-level restatement (oracle.two_level_trace): with
identity instance transforms the object-space rays are the world rays bit for bit, so it
must give exactly the flattened oracle's closest and any hits; with real transforms it
must agree with the flattened oracle on rays that stay clear of triangle edges."""
import json

import numpy as np

import oracle
from btrc_gb300 import scenes
from oracle import scene as OS


def _identity_scene(out):
    out.mkdir(parents=True, exist_ok=True)
    rng = np.random.default_rng(4)
    c = rng.uniform(-1, 1, (400, 3))
    v = c[:, None, :] + rng.normal(0, 0.1, (400, 3, 3))
    scenes.write_obj(out / "soup.obj", v.reshape(-1, 3), np.arange(1200).reshape(-1, 3))
    qv, qf = scenes.quad(4.0)
    scenes.write_obj(out / "ground.obj", qv, qf)
    ent = lambda fn: {"geometry": {"type": "triangle_mesh", "filename": "$env{scene_directory}/" + fn},
                      "material": {"type": "diffuse", "color": [0.5, 0.5, 0.5]}}
    scene = {"width": 16, "height": 16,
             "camera": {"type": "pinhole", "eye": [0.0, 0.0, 4.0], "dst": [0.0, 0.0, 0.0], "up": [0.0, 1.0, 0.0],
                        "fov_y": {"deg": 50.0}},
             "renderer": {"type": "wfpt", "spp": 1},
             "scene": {"entities": [ent("soup.obj"), ent("soup.obj"), ent("ground.obj")]}}
    p = out / "scene.json"
    p.write_text(json.dumps(scene))
    return p


def _rays(n, seed):
    rng = np.random.default_rng(seed)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(-2, 2, (n, 3))
    rays[:, 4:7] = rng.normal(size=(n, 3))
    rays[:, 7] = 3.0e38
    rays[n // 3:n // 2, 7] = 1.0
    return rays


def test_two_level_oracle_equals_flattened_under_identity(tmp_path):
    S = OS.Scene(_identity_scene(tmp_path / "ident"))
    rays = _rays(3000, 1)
    f2, h2, o2 = oracle.two_level_trace(S, rays)
    bvh = oracle.OracleBvh(S.tris, S.ids)
    f1, h1 = bvh.closest(rays)
    o1 = bvh.any(rays)
    assert np.array_equal(f1, f2)
    hit = f1 != 0
    assert hit.mean() > 0.2
    assert np.array_equal(h1[hit].view(np.uint32), h2[hit].view(np.uint32))
    assert np.array_equal(o1, o2)
    # two instances of one mesh at the same place: ties at equal t go to the lower instance
    assert (f1[hit] & 0x3FFFFFFF).max() <= 2


def test_two_level_oracle_matches_flattened_with_transforms(tmp_path):
    path = scenes.random_soup(tmp_path / "soup", seed=5, n_tris=3000, n_instances=4)
    S = OS.Scene(path)
    rays = _rays(3000, 2)
    f2, h2, o2 = oracle.two_level_trace(S, rays)
    bvh = oracle.OracleBvh(S.tris, S.ids)
    f1, h1 = bvh.closest(rays)
    # object-space and world-space arithmetic round differently, so only hits away from
    # edges and near-ties must agree: the same triangle for nearly every ray, and t
    # close to the world-space t
    same = f1 == f2
    assert same.mean() > 0.995
    both = same & (f1 != 0)
    rel = np.abs(h1[both, 0] - h2[both, 0]) / np.abs(h1[both, 0])
    assert np.percentile(rel, 99) < 1e-5 and rel.max() < 1e-3  # grazing hits amplify rounding
    assert np.array_equal(h1[both, 1].view(np.uint32), h2[both, 1].view(np.uint32))
