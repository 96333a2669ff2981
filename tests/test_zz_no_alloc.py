"""btrc_render_noalloc: rendering without allocating GPU memory during the call.

Some callers cannot call cudaMalloc while they render (engines that reserve all device
memory up front, processes under a hard memory budget, latency-critical threads where
cudaMalloc/cudaFree would synchronise the device). For them the library keeps the
render's scratch in one fixed device array. This file is collected last so that a run
stopping at the first failure has run every other test first; it builds its own
context and scene, so it also passes alone in a fresh process."""
import json

import numpy as np
import pytest

import btrc_gb300 as B
from btrc_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(native_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = B.Context(0)
    yield c
    c.close()


def test_noalloc_matches_render_on_two_calls(ctx, tmp_path):
    import torch
    path = scenes.cornell(out_dir=tmp_path / "cornell", width=64, height=64, spp=16)
    sc = ctx.load_scene(path).build()
    want = ctx.render(sc)  # the regular entry point, host output
    out = torch.empty((64, 64, 3), dtype=torch.float32, device="cuda")
    for call in range(2):
        out.fill_(-1.0)  # every pixel must be written by the call
        torch.cuda.synchronize()  # the fill is done before the render reads or writes out
        free_before = torch.cuda.mem_get_info()[0]
        stats = {}
        ctx.render_noalloc(sc, out, stats=stats)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        got = out.cpu().numpy()
        assert stats["paths"] == 64 * 64 * 16 and stats["traversal_errors"] == 0, (call, stats)
        # same tolerance as the render-vs-render determinism test (atomic summation order)
        assert np.allclose(got, want, rtol=1e-4, atol=1e-5), (call, np.abs(got - want).max())
        if call == 1:
            # the first call may load kernel modules (and with them the fixed array); the
            # second must leave the device's free memory exactly where it was
            assert free_after == free_before, (free_before, free_after)
    sc.close()


def test_noalloc_rejects_a_short_output(ctx, tmp_path):
    import torch
    path = scenes.cornell(out_dir=tmp_path / "short", width=32, height=32, spp=1)
    sc = ctx.load_scene(path).build()
    with pytest.raises(B.BtrcError) as e:
        ctx.render_noalloc(sc, torch.empty((32 * 32 * 3 - 1,), dtype=torch.float32, device="cuda"))
    assert e.value.status == 1
    sc.close()


def test_noalloc_rejects_films_beyond_its_scratch(ctx, tmp_path):
    import torch
    path = scenes.cornell(out_dir=tmp_path / "big", width=600, height=600, spp=1)
    sc = ctx.load_scene(path).build()
    out = torch.empty((600, 600, 3), dtype=torch.float32, device="cuda")
    with pytest.raises(B.BtrcError) as e:
        ctx.render_noalloc(sc, out)
    assert e.value.status == 1 and "262144" in str(e.value)
    sc.close()
