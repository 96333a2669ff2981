"""CPU tests of the C ABI surface and the scene loader (host-only context, no GPU).

The loader must accept Btrc's scene schema with its quirks: scalars pass through
std::to_string(float) (six decimals), "$include{}" splices text, "$reference{}" shares one
node (so one geometry / one material object), transform arrays compose later elements on
the left, and errors come back as status codes with a message."""
import json
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import btrc_gb300 as B
from btrc_gb300 import scenes
from oracle import scene as OS

ROOT = Path(__file__).resolve().parent.parent


def test_library_exports_every_declared_symbol(native_lib):
    header = (ROOT / "include" / "btrc.h").read_text()
    declared = set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(btrc_[a-z_0-9]+)\s*\(", header, re.M))
    assert len(declared) >= 18
    out = subprocess.run(["nm", "-D", "--defined-only", str(B.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (btrc_[a-z_0-9]+)$", out, re.M))
    missing = declared - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    # the Python mirror binds every declared entry point
    assert declared <= set(B.SIGNATURES)


def test_version_string(native_lib):
    assert "sm_103a" in B.version()


def _write(tmp, name, obj):
    p = Path(tmp) / name
    p.write_text(json.dumps(obj) if not isinstance(obj, str) else obj)
    return p


def _minimal(tmp, extra_entities=(), renderer=None, **root):
    v, f = scenes.quad(2.0)
    scenes.write_obj(Path(tmp) / "q.obj", v, f)
    ents = [{"geometry": {"type": "triangle_mesh", "filename": "$env{scene_directory}/q.obj"},
             "material": {"type": "diffuse", "color": [0.5, 0.5, 0.5]}}] + list(extra_entities)
    scene = {"width": 8, "height": 6,
             "camera": {"type": "pinhole", "eye": [0, 1, 3], "dst": [0, 0, 0], "up": [0, 1, 0], "fov_y": {"deg": 45}},
             "renderer": renderer or {"type": "wfpt", "spp": 2},
             "scene": {"entities": ents}}
    scene.update(root)
    return scene


def test_host_only_context_loads_and_builds(native_lib, tmp_path):
    p = _write(tmp_path, "s.json", _minimal(tmp_path))
    ctx = B.Context(-1)
    sc = ctx.load_scene(p).build()
    info = sc.info()
    assert (info.width, info.height, info.spp, info.triangles) == (8, 6, 2, 2)
    with pytest.raises(B.BtrcError) as e:
        ctx.render(sc)
    assert e.value.status == 1 and "host-only" in str(e.value)
    # host-only contexts build the flattened form whatever the options ask for
    sc2 = ctx.load_scene(p).build(two_level=True)
    assert sc2.info().two_level == 0 and sc2.info().bvh_nodes == info.bvh_nodes


@pytest.mark.parametrize("content,status", [
    ("{ not json", 3),
    ('{"width": 8}', 3),
])
def test_parse_errors(native_lib, tmp_path, content, status):
    p = _write(tmp_path, "bad.json", content)
    ctx = B.Context(-1)
    with pytest.raises(B.BtrcError) as e:
        ctx.load_scene(p)
    assert e.value.status == status


def test_missing_file_is_io_error(native_lib, tmp_path):
    ctx = B.Context(-1)
    with pytest.raises(B.BtrcError) as e:
        ctx.load_scene(tmp_path / "nope.json")
    assert e.value.status == 2
    s = _minimal(tmp_path)
    s["scene"]["entities"][0]["geometry"]["filename"] = "$env{scene_directory}/missing.obj"
    with pytest.raises(B.BtrcError) as e:
        ctx.load_scene(_write(tmp_path, "m.json", s))
    assert e.value.status == 2


def test_unsupported_material_is_reported(native_lib, tmp_path):
    s = _minimal(tmp_path)
    s["scene"]["entities"][0]["material"] = {"type": "velvet"}
    ctx = B.Context(-1)
    with pytest.raises(B.BtrcError) as e:
        ctx.load_scene(_write(tmp_path, "u.json", s))
    assert e.value.status == 8 and "velvet" in str(e.value)


def test_bad_reference_is_parse_error(native_lib, tmp_path):
    s = _minimal(tmp_path)
    s["scene"]["entities"].append({"geometry": "$reference{$root/scene/entities/7/geometry}",
                                   "material": {"type": "diffuse", "color": 0.5}})
    ctx = B.Context(-1)
    with pytest.raises(B.BtrcError) as e:
        ctx.load_scene(_write(tmp_path, "r.json", s))
    assert e.value.status == 3


def test_reference_shares_geometry_and_include_splices(native_lib, tmp_path):
    s = _minimal(tmp_path, extra_entities=[
        {"geometry": "$reference{$root/scene/entities/0/geometry}", "material": "$include{mat.json}",
         "local_to_world": [{"scale": [0.5, 1, 0.5]}, {"translate": [0, 1, 0]}]}])
    (tmp_path / "mat.json").write_text('{"type": "diffuse", "color": [0.2, 0.3, 0.4]}')
    text = json.dumps(s).replace('"$include{mat.json}"', '"$include{mat.json}"')
    p = _write(tmp_path, "ref.json", text)
    ctx = B.Context(-1)
    sc = ctx.load_scene(p).build()
    info = sc.info()
    assert info.geometries == 1 and info.instances == 2 and info.materials == 2 and info.triangles == 4
    xyz, ids = sc.export_triangles()
    S = OS.Scene(p)
    assert np.array_equal(xyz.view(np.uint32), S.tris.view(np.uint32))


def test_scalars_pass_through_to_string(native_lib, tmp_path):
    # 1e-7 becomes "0.000000" in the reference's node tree, i.e. zero
    s = _minimal(tmp_path, extra_entities=[
        {"geometry": "$reference{$root/scene/entities/0/geometry}", "material": {"type": "diffuse", "color": 0.5},
         "local_to_world": {"translate": [1e-7, 0.1234567, 2.5]}}])
    p = _write(tmp_path, "f.json", s)
    ctx = B.Context(-1)
    xyz, _ = ctx.load_scene(p).build().export_triangles()
    quad = scenes.quad(2.0)[0]
    moved = xyz[2:].reshape(-1, 3)
    assert np.all(moved[:, 0] == np.float32(np.float32(quad[[0, 2, 1, 0, 3, 2], 0])))  # x unchanged
    assert np.all(moved[:, 1] == np.float32(0.123457))


def test_rotation_transforms_match_oracle(native_lib, tmp_path):
    s = _minimal(tmp_path, extra_entities=[
        {"geometry": "$reference{$root/scene/entities/0/geometry}", "material": {"type": "diffuse", "color": 0.5},
         "local_to_world": [{"rotate": {"axis": [1, 2, 3], "angle": {"deg": 33}}}, {"rotate_x": {"deg": 20}},
                            {"rotate_y": {"rad": 0.3}}, {"rotate_z": {"deg": 10}}, {"translate": [0.5, 0, 0]}]}])
    p = _write(tmp_path, "rot.json", s)
    ctx = B.Context(-1)
    xyz, _ = ctx.load_scene(p).build().export_triangles()
    S = OS.Scene(p)
    # sin/cos come from two different libm implementations: allow a few ulps
    assert np.allclose(xyz, S.tris, rtol=0, atol=4e-7)


def test_wfpt_defaults_and_pt_renderer(native_lib, tmp_path):
    s = _minimal(tmp_path, renderer={"type": "pt"})
    ctx = B.Context(-1)
    info = ctx.load_scene(_write(tmp_path, "pt.json", s)).info()
    # WavefrontPathTracer::Params defaults (builtin/btrc/builtin/renderer/wavefront.h:13-27)
    assert (info.spp, info.min_depth, info.max_depth, info.state_count) == (128, 5, 10, 1000000)
    assert info.sampler == 0 and info.filter == 0


def test_post_processors_parse(native_lib, tmp_path):
    # a group or an array of post processors (factory/btrc/factory/post_processor.cpp:5-25);
    # unknown types fail to load, denoise loads
    base = json.loads(scenes.cornell(out_dir=tmp_path, width=8, height=8, spp=1).read_text())
    ctx = B.Context(-1)
    for post, ok in (({"type": "tonemap"}, True),
                     ([{"type": "tonemap", "exposure": 2}, {"type": "save", "color": "x.png"}], True),
                     ([{"type": "denoise"}], True),
                     ([{"type": "blur"}], False),
                     ("tonemap", False)):
        sc = dict(base)
        sc["post_processors"] = post
        q = tmp_path / "p.json"
        q.write_text(json.dumps(sc))
        if ok:
            ctx.load_scene(q)
        else:
            with pytest.raises(B.BtrcError):
                ctx.load_scene(q)
    ctx.close()


def _procedural_scene(tmp_path):
    scene = {"width": 32, "height": 32,
             "camera": {"type": "pinhole", "eye": [0, 1, 3], "dst": [0, 0, 0], "up": [0, 1, 0], "fov_y": {"deg": 40}},
             "renderer": {"type": "wfpt", "spp": 4},
             "scene": {"entities": [
                 {"geometry": {"type": "sphere", "subdivisions": 2}, "material": {"type": "diffuse", "color": 0.7},
                  "local_to_world": [{"scale": 0.4}, {"translate": [-0.5, 0.4, 0]}]},
                 {"geometry": {"type": "quad"}, "material": {"type": "diffuse", "color": [0.8, 0.6, 0.4]},
                  "local_to_world": {"scale": 4}},
                 {"geometry": {"type": "box"}, "material": {"type": "metal", "color": 0.9, "roughness": 0.3},
                  "local_to_world": [{"rotate_y": {"deg": 30}}, {"translate": [0.6, 0.5, 0]}]},
                 {"geometry": {"type": "quad"}, "material": {"type": "diffuse", "color": 0.0},
                  "local_to_world": [{"rotate_x": {"deg": 180}}, {"scale": 0.5}, {"translate": [0, 2, 0]}],
                  "light": {"type": "mesh_light", "intensity": 8}}]}}
    p = tmp_path / "proc.json"
    p.write_text(json.dumps(scene))
    return p


def test_procedural_geometry_matches_oracle(native_lib, tmp_path):
    # inline "sphere" / "quad" / "box" creators: the loader's flattened world triangles
    # equal the oracle's construction bit for bit
    p = _procedural_scene(tmp_path)
    ctx = B.Context(-1)
    sc = ctx.load_scene(p).build()
    xyz, ids = sc.export_triangles()
    S = OS.Scene(p)
    assert len(xyz) == len(S.tris) == 320 + 2 + 12 + 2
    order_o = np.lexsort((S.ids[:, 1], S.ids[:, 0]))
    order_p = np.lexsort((ids[:, 1], ids[:, 0]))
    assert np.array_equal(ids[order_p], S.ids[order_o])
    assert np.array_equal(xyz[order_p].view(np.uint32), S.tris[order_o].view(np.uint32))
    ctx.close()


def test_render_noalloc_rejects_host_or_short_outputs(native_lib, tmp_path):
    """k_resolve writes H*W*3 floats through the allocation-free entry point's output
    pointer, so the Python mirror refuses anything but a large enough float32 CUDA tensor
    before the library is called (no launch happens; a host-only context suffices)."""
    torch = pytest.importorskip("torch")
    p = _write(tmp_path, "s.json", _minimal(tmp_path))
    ctx = B.Context(-1)
    sc = ctx.load_scene(p).build()
    for bad in (np.zeros((6, 8, 3), np.float32), torch.zeros((6, 8, 3), dtype=torch.float32)):
        with pytest.raises(B.BtrcError) as e:
            ctx.render_noalloc(sc, bad)
        assert e.value.status == 1 and "CUDA tensor" in str(e.value)
    sc.close()
    ctx.close()


def test_scenes_load_build_matches_one_by_one(native_lib, scene_dir):
    """btrc_scenes_load_build loads and builds several scenes on one shared pool of host
    threads; each scene's BVH is the one a single load and build gives (the build does not
    depend on the threads it gets), and a missing file fails the whole call with IO."""
    paths = scenes.batch(count=5, seed=79, out_dir=scene_dir / "batch-load")
    ctx = B.Context(-1)
    many = ctx.load_build_scenes(paths)
    for p, sc in zip(paths, many):
        one = ctx.load_scene(p).build()
        a, b = sc.info(), one.info()
        assert (a.triangles, a.bvh_nodes, a.bvh_bytes, a.width, a.height) == \
            (b.triangles, b.bvh_nodes, b.bvh_bytes, b.width, b.height)
        na, ta = sc.export_bvh()
        nb, tb = one.export_bvh()
        assert np.array_equal(na, nb)
        one.close()
        sc.close()
    with pytest.raises(B.BtrcError) as e:
        ctx.load_build_scenes([paths[0], str(Path(paths[0]).parent / "missing.json")])
    assert e.value.status == 2
    ctx.close()
