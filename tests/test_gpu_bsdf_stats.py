"""Statistical checks of the GPU BSDF kernels that do not compare with the oracle.

Through btrc_bsdf_batch (op 2: the sampled direction before Disney's bad-sample
rejection, op 0: f and pdf) on the GB300:
  * chi-square: the sampled directions follow pdf (3 M samples per case, every lobe of
    diffuse, the GGX conductor and Disney; Disney's transmission pdf corrected by the
    factor the reference's own sampler needs, see tests/bsdf_stats.py);
  * the importance-sampled and the uniformly sampled directional albedo agree;
  * white furnace: a white Lambertian returns exactly 1 per sample, a white conductor
    (R0 = 1) and a white metallic Disney surface at most 1.
Each pins the kernel's sampling and evaluation against each other and against
physical bounds, independently of the CPU restatement."""
import numpy as np
import pytest

from tests import bsdf_stats as S

pytestmark = pytest.mark.gpu
pytest.importorskip("scipy")


def _hook(ctx, op):
    import torch

    def run(m, wo, wu):
        n = len(m)
        out = torch.zeros((n, 4 if op == 0 else 7), dtype=torch.float32, device="cuda")
        ctx.bsdf_batch(op, torch.from_numpy(np.ascontiguousarray(m, np.float32)).cuda(),
                       torch.from_numpy(np.ascontiguousarray(wo, np.float32)).cuda(),
                       torch.from_numpy(np.ascontiguousarray(wu, np.float32)).cuda(), n, out)
        torch.cuda.synchronize()
        return out.cpu().numpy().astype(np.float64)
    return run


@pytest.mark.parametrize("name,mat,theta", S.CASES, ids=[c[0] for c in S.CASES])
def test_gpu_sampling_density_matches_pdf(gpu_ctx, name, mat, theta):
    sample, ev = _hook(gpu_ctx, 2), _hook(gpu_ctx, 0)
    wo = S.direction(theta).astype(np.float32).astype(np.float64)
    p, stat, dof, drawn = S.chi_square(sample, ev, mat, wo, n=3_000_000, seed=21)
    assert p > 1e-4, (name, p, stat, dof, drawn)
    (a, sa), (b, sb), _ = S.albedo_two_ways(sample, ev, mat, wo, n=1_000_000, seed=22)
    assert np.all(np.abs(a - b) < 5 * np.hypot(sa, sb) + 1e-5), (name, a, sa, b, sb)


def test_gpu_white_furnace(gpu_ctx):
    sample, ev = _hook(gpu_ctx, 2), _hook(gpu_ctx, 0)
    wo = S.direction(40.0).astype(np.float32).astype(np.float64)
    (a, _), _, v = S.albedo_two_ways(sample, ev, S.material("diffuse", color=1.0), wo, n=500_000)
    assert np.allclose(v, 1.0, rtol=2e-6), np.abs(v - 1).max()
    for mat in (S.material("metal", color=1.0, roughness=0.4),
                S.material("disney", color=1.0, metallic=1.0, roughness=0.4, specular=0.5)):
        (a, sa), _, _ = S.albedo_two_ways(sample, ev, mat, wo, n=1_000_000)
        assert np.all(a <= 1.0 + 4 * sa), (a, sa)
        assert np.all(a > 0.8), a
