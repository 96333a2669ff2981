"""The statistical BSDF checks (tests/bsdf_stats.py) on the FP64 oracle, on the CPU.

They hold for the oracle's restatement of the reference's materials (with the
transmission-pdf correction that the reference's own sampler needs), and they have the
power to see a wrong pdf: the same chi-square rejects a pdf changed by a few percent on
one lobe (a mistake planted in the oracle's output, here on the CPU)."""
import numpy as np
import pytest

import oracle
from tests import bsdf_stats as S

pytest.importorskip("scipy")


def _sample(m, wo, u):
    return oracle.bsdf_batch(2, m, wo, u)


def _eval(m, wo, wi):
    return oracle.bsdf_batch(0, m, wo, wi)


@pytest.mark.parametrize("name,mat,theta", S.CASES, ids=[c[0] for c in S.CASES])
def test_oracle_sampling_density_matches_pdf(oracle_lib, name, mat, theta):
    wo = S.direction(theta)
    p, stat, dof, drawn = S.chi_square(_sample, _eval, mat, wo, n=1_000_000, seed=11)
    assert p > 1e-4, (name, p, stat, dof)
    (a, sa), (b, sb), _ = S.albedo_two_ways(_sample, _eval, mat, wo, n=300_000, seed=12)
    assert np.all(np.abs(a - b) < 5 * np.hypot(sa, sb) + 1e-6), (name, a, sa, b, sb)


def test_chi_square_sees_a_wrong_pdf(oracle_lib):
    """A pdf 4 % too high on the upper half of the specular lobe's half-vector range."""
    name, mat, theta = S.CASES[2]  # metal r0.3

    def bad_eval(m, wo, wi):
        out = _eval(m, wo, wi)
        h = wo + wi
        h /= np.maximum(np.linalg.norm(h, axis=1, keepdims=True), 1e-12)
        out[:, 3] *= np.where(h[:, 2] > 0.97, 1.04, 1.0)
        return out

    p, stat, dof, _ = S.chi_square(_sample, bad_eval, mat, S.direction(theta), n=1_000_000, seed=11)
    assert p < 1e-6, (p, stat, dof)


def test_oracle_white_furnace(oracle_lib):
    wo = S.direction(40.0)
    (a, _), _, v = S.albedo_two_ways(_sample, _eval, S.material("diffuse", color=1.0), wo, n=100_000)
    assert np.allclose(v, 1.0, rtol=1e-12)
    for mat in (S.material("metal", color=1.0, roughness=0.4),
                S.material("disney", color=1.0, metallic=1.0, roughness=0.4, specular=0.5)):
        (a, sa), _, _ = S.albedo_two_ways(_sample, _eval, mat, wo, n=300_000)
        assert np.all(a <= 1.0 + 4 * sa), (a, sa)
        assert np.all(a > 0.8), a
