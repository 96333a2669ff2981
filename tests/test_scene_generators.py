"""Seeded scene generators: the cached scene file follows every renderer setting it is
asked for (a cached file written for another queue length must not be reused)."""
import json

from btrc_gb300 import scenes


def test_cornell_cache_is_keyed_by_state_count(tmp_path):
    a = scenes.cornell(out_dir=tmp_path, width=16, height=16, spp=2, state_count=1000000)
    b = scenes.cornell(out_dir=tmp_path, width=16, height=16, spp=2)
    assert a != b
    assert json.loads(a.read_text())["renderer"]["state_count"] == 1000000
    assert json.loads(b.read_text())["renderer"]["state_count"] == 32 * 1024 * 1024
    # asking again returns the cached file unchanged
    assert scenes.cornell(out_dir=tmp_path, width=16, height=16, spp=2, state_count=1000000) == a


def test_terrain_cache_is_keyed_by_state_count(tmp_path):
    a = scenes.terrain(out_dir=tmp_path, width=16, height=9, spp=1, grid=16, instances=2, state_count=1 << 20)
    b = scenes.terrain(out_dir=tmp_path, width=16, height=9, spp=1, grid=16, instances=2, state_count=1 << 22)
    assert a != b
    assert json.loads(a.read_text())["renderer"]["state_count"] == 1 << 20
    assert json.loads(b.read_text())["renderer"]["state_count"] == 1 << 22
