"""Volume primitives (scene `volumes[]`) in the oracle, on the CPU.

The oracle restates VolumePrimitiveMedium (core/btrc/core/volume.cpp:112-197): the segment
is walked from one box boundary to the next and ratio tracking runs inside each overlap
region with the summed majorant of the boxes there (core/btrc/core/volume/aggregate.cpp:
221-252). Ratio tracking is unbiased, so through constant-density boxes the mean estimate
must be exp(-integral of the summed sigma_t)."""
from pathlib import Path

import numpy as np
import pytest

from btrc_gb300 import scenes
from oracle import scene as OS


@pytest.fixture(scope="module")
def fog(tmp_path_factory):
    out = tmp_path_factory.mktemp("fog")
    return OS.Scene(scenes.cornell(out_dir=out, width=16, height=16, spp=4, variant="fog"))


def _mean_tr(S, a, b, n=40000):
    seg = np.tile(np.array([a + b], np.float32), (n, 1))
    tr = S.medium_tr(S.vacuum, seg, np.arange(n, dtype=np.uint64) * 7919 + 3).astype(np.float64)
    return tr.mean(), tr.std() / np.sqrt(n)


def test_volume_medium_is_last_and_bounds_include_boxes(fog):
    assert fog.nvol == 3
    assert fog.vacuum == len(fog.med) - 1 and fog.med[fog.vacuum][0] == 3
    # the reference bounds a volume by o, o + x, o + y, o + z only (volume.cpp:54-68)
    lo, hi = OS.volume_box(fog.vol[1])
    assert np.allclose(lo, [-0.25, -0.35, 0.4], atol=1e-6) and np.allclose(hi, [0.3, 0.1, 0.9], atol=1e-6)


def test_single_constant_box(fog):
    # inside box 0 only (sigma_t 2): x from -0.44 to -0.2 at y = z = -0.4 + 0.7 offset
    m, se = _mean_tr(fog, [-0.44, -0.4, 0.3], [-0.2, -0.4, 0.3])
    assert abs(m - np.exp(-2.0 * 0.24)) < 4 * se + 1e-4, (m, se)


def test_overlap_of_two_constant_boxes(fog):
    # y = 0.03, z = 0.32 crosses box 0 (sigma 2, x in [-0.45, 0.1]) and box 2 (sigma 1,
    # x in [-0.3, 0.3]) but not the sheared grid box (z >= 0.4 there)
    a, b = [-0.44, 0.03, 0.32], [0.28, 0.03, 0.32]
    m, se = _mean_tr(fog, a, b)
    want = np.exp(-(2.0 * 0.54 + 1.0 * 0.58))
    assert abs(m - want) < 4 * se + 1e-4, (m, want, se)
    # the reverse direction walks the same boxes
    m2, se2 = _mean_tr(fog, b, a)
    assert abs(m2 - want) < 4 * se2 + 1e-4, (m2, want, se2)


def test_segment_outside_all_boxes_is_clear(fog):
    m, _ = _mean_tr(fog, [0.35, 0.4, -0.4], [0.45, -0.4, -0.45], n=100)
    assert m == 1.0


def test_byte_text_grid_reads_characters(tmp_path):
    # "byte" components are single characters, read as signed 8-bit normalised values
    (tmp_path / "g.txt").write_text("byte 1 2 1 1\n" + chr(127) + chr(64) + "\n")
    from oracle.scene import _grid, _to_node
    _c, g = _grid(_to_node({"type": "array", "text": str(tmp_path / "g.txt")}), str(tmp_path))
    assert np.allclose(g.ravel(), [1.0, 64 / 127.0])


def test_oracle_ratio_tracking_linear_grid(tmp_path):
    """The oracle's heterogeneous-medium ratio tracking (builtin/btrc/builtin/medium/
    hetergeneous.cpp:75-106) behind a transform medium: along a density linear in x, y
    and z its mean estimate is exp(-length * sigma(midpoint))."""
    from tests.util import ramp_medium_scene, ramp_segments, ramp_tr_exact
    S = OS.Scene(ramp_medium_scene(tmp_path))
    n = 60000
    for s in ramp_segments():
        seg = np.tile(s.astype(np.float32), (n, 1))
        tr = S.medium_tr(0, seg, np.arange(n, dtype=np.uint64) * 7919 + 3).astype(np.float64)
        want = float(ramp_tr_exact(s.astype(np.float32).astype(np.float64)))
        assert abs(tr.mean() - want) < 4.5 * tr.std() / np.sqrt(n), (s, tr.mean(), want)
