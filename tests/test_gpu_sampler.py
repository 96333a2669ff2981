"""Sampler streams on the GPU, bit-exact against the oracle (integer and exactly rounded
FP32 arithmetic only)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,width,height", [(0, 256, 256), (1, 256, 256), (1, 1920, 1080), (1, 7, 5), (0, 1920, 1080)])
def test_sampler_bitexact(gpu_ctx, kind, width, height):
    import torch
    rng = np.random.default_rng(kind * 100 + width)
    n, dims = 4096, 40
    px = rng.integers(0, width, n).astype(np.uint32)
    py = rng.integers(0, height, n).astype(np.uint32)
    pix = px | (py << 16)
    s = rng.integers(0, 4096, n).astype(np.uint32)
    out = torch.zeros((n, dims), dtype=torch.float32, device="cuda")
    gpu_ctx.sampler_batch(kind, width, height, torch.from_numpy(pix.view(np.int32)).cuda(),
                          torch.from_numpy(s.view(np.int32)).cuda(), n, dims, out)
    torch.cuda.synchronize()
    ref = oracle.sampler_batch(kind, width, height, pix, s, dims)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref.view(np.uint32))


def test_halton_dimension_wrap(gpu_ctx):
    # more than 1000 dimensions wraps back to dimension 2 (halton.cpp:82-91)
    import torch
    n, dims = 64, 1100
    pix = np.arange(n, dtype=np.uint32)
    s = np.zeros(n, np.uint32)
    out = torch.zeros((n, dims), dtype=torch.float32, device="cuda")
    gpu_ctx.sampler_batch(1, 64, 64, torch.from_numpy(pix.view(np.int32)).cuda(),
                          torch.from_numpy(s.view(np.int32)).cuda(), n, dims, out)
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    ref = oracle.sampler_batch(1, 64, 64, pix, s, dims)
    assert np.array_equal(o.view(np.uint32), ref.view(np.uint32))
    # output k is dimension 2 + k up to k = 997; k = 998 wraps back to dimension 2
    assert np.array_equal(o[:, 998:1096], o[:, 0:98])
