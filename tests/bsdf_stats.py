"""Statistical BSDF checks that need no second implementation of the BSDF.

Each check uses only the implementation under test: its sampler (the direction drawn
from (wo, u), before Disney's bad-sample rejection) and its eval / pdf. They pin
properties the reference's material code must have whatever its formulas are
(builtin/btrc/builtin/material/disney.cpp:477-730, material/component/diffuse.cpp,
material/component/microfacet_reflection.h):

  * chi-square: the density of the sampled directions equals pdf(wi) (histogram over
    equal-solid-angle bins of the sphere against pdf integrated over each bin);
  * two estimators of the directional albedo int f |cos| dwi agree: importance sampled,
    f |cos| / pdf at the sampler's own directions, and uniform over the sphere, 4 pi f |cos|;
  * white furnace: a white Lambertian reflects exactly 1, a white (R0 = 1) conductor and a
    white metallic Disney surface at most 1.

`sample(mat, wo, u)` returns (n, 7) rows (drawn, 0, 0, 0, wi.xyz) and
`eval_fp(mat, wo, wi)` returns (n, 4) rows (f.rgb, pdf), both in float64 numpy.
"""
from __future__ import annotations

import numpy as np

TWO_PI = 2.0 * np.pi


def material(kind: str, **p) -> np.ndarray:
    """One 16-float material record in the layout of btrc_bsdf_batch (type in [15])."""
    m = np.zeros(16, np.float32)
    if kind == "diffuse":
        m[0:3] = p.get("color", 0.8)
        m[15] = 0
    elif kind == "metal":
        m[0:3] = p.get("color", 0.9)
        m[3] = p["roughness"]
        m[4] = p.get("anisotropic", 0.0)
        m[15] = 1
    else:
        m[0:3] = p.get("color", 0.7)
        m[3] = p.get("metallic", 0.0)
        m[4] = p["roughness"]
        m[5] = p.get("specular", 0.5)
        m[6] = p.get("specular_tint", 0.0)
        m[7] = p.get("anisotropic", 0.0)
        m[8] = p.get("sheen", 0.0)
        m[9] = p.get("sheen_tint", 0.0)
        m[10] = p.get("clearcoat", 0.0)
        m[11] = p.get("clearcoat_gloss", 1.0)
        m[12] = p.get("transmission", 0.0)
        m[13] = p.get("transmission_roughness", p["roughness"])
        m[14] = p.get("ior", 1.5)
        m[15] = 2
    return m


def direction(theta_deg: float, phi: float = 0.3) -> np.ndarray:
    t = np.radians(theta_deg)
    return np.array([np.sin(t) * np.cos(phi), np.sin(t) * np.sin(phi), np.cos(t)])


def transmission_density_factor(mat, wo, wi):
    """Ratio of the transmission lobe's true sampling density to the pdf the reference
    reports for it, per direction (1 off the transmission side).

    DisneyBSDF::sample_transmission (disney.cpp:277-308) draws the half vector with density
    D(h) cos(theta_h) and refracts wo about it, so the density of wi is
    D(h) cos(theta_h) |dh/dwi|. pdf_transmission (disney.cpp:369-404) returns
    |wi.h| D(h) |dh/dwi| instead: cos(theta_h) is replaced by |wi.h|. A faithful
    restatement keeps that pdf (it sets the MIS weights and f |cos| / pdf of every
    transmission sample), so the checks compare the sampler with the true density,
    pdf * cos(theta_h) / |wi.h|, on the transmission side."""
    wi = np.asarray(wi, np.float64)
    wo = np.broadcast_to(np.asarray(wo, np.float64), wi.shape)
    if mat[15] != 2 or mat[12] == 0.0:
        return np.ones(len(wi))
    ior = float(mat[14])
    eta = np.where(wo[:, 2] > 0, ior, 1.0 / ior)
    h = wo + eta[:, None] * wi
    h = h / np.linalg.norm(h, axis=1, keepdims=True)
    h = np.where(h[:, 2:3] < 0, -h, h)
    widoth = np.abs((wi * h).sum(1))
    trans = wi[:, 2] * wo[:, 2] < 0
    with np.errstate(divide="ignore", invalid="ignore"):
        f = np.where(trans & (widoth > 0), h[:, 2] / widoth, 1.0)
    return f


def _tile(mat, wo, n):
    return np.tile(mat, (n, 1)), np.tile(np.asarray(wo, np.float64), (n, 1))


def chi_square(sample, eval_fp, mat, wo, n=2_000_000, seed=0, n_cos=24, n_phi=48, sub=12):
    """Chi-square test of the sampled directions against pdf. Bins are equal-solid-angle
    cells of (cos theta, phi); each bin's expected count is n times pdf integrated over
    the cell by the sub x sub midpoint rule. Samples that draw no direction form one more
    category, expected n (1 - sum of the integrals). Cells expected below 5 are pooled.
    Returns (p value, statistic, degrees of freedom, fraction of samples drawn)."""
    from scipy import stats
    rng = np.random.default_rng(seed)
    mats, wos = _tile(mat, wo, n)
    out = sample(mats, wos, rng.random((n, 3)))
    drawn = out[:, 0] > 0
    d = out[drawn, 4:7]
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    ct = np.clip(d[:, 2], -1.0, 1.0)
    ph = np.mod(np.arctan2(d[:, 1], d[:, 0]), TWO_PI)
    it = np.minimum(((ct + 1.0) * 0.5 * n_cos).astype(np.int64), n_cos - 1)
    ip = np.minimum((ph / TWO_PI * n_phi).astype(np.int64), n_phi - 1)
    obs = np.bincount(it * n_phi + ip, minlength=n_cos * n_phi).astype(np.float64)

    # midpoint points of every cell
    a = (np.arange(sub) + 0.5) / sub
    ci = (np.arange(n_cos)[:, None] + a[None, :]) * (2.0 / n_cos) - 1.0      # (n_cos, sub)
    pj = (np.arange(n_phi)[:, None] + a[None, :]) * (TWO_PI / n_phi)         # (n_phi, sub)
    C = np.broadcast_to(ci[:, None, :, None], (n_cos, n_phi, sub, sub)).reshape(-1)
    P = np.broadcast_to(pj[None, :, None, :], (n_cos, n_phi, sub, sub)).reshape(-1)
    s = np.sqrt(np.maximum(0.0, 1.0 - C * C))
    wi = np.stack([s * np.cos(P), s * np.sin(P), C], 1)
    m2, wo2 = _tile(mat, wo, len(wi))
    pdf = eval_fp(m2, wo2, wi)[:, 3] * transmission_density_factor(mat, wo, wi)
    pdf = np.where(np.isfinite(pdf), pdf, 0.0)
    cell = (2.0 / n_cos) * (TWO_PI / n_phi)
    integral = pdf.reshape(n_cos * n_phi, sub * sub).mean(1) * cell
    exp = n * integral

    obs_all = np.concatenate([obs, [n - drawn.sum()]])
    exp_all = np.concatenate([exp, [max(n - exp.sum(), 0.0)]])
    # pool small cells (and any cell with no expectation) into one category
    small = exp_all < 5.0
    o = np.concatenate([obs_all[~small], [obs_all[small].sum()]])
    e = np.concatenate([exp_all[~small], [exp_all[small].sum()]])
    if e[-1] < 5.0:  # the pooled remainder itself too small: fold it into the largest cell
        k = int(np.argmax(e[:-1]))
        o[k] += o[-1]
        e[k] += e[-1]
        o, e = o[:-1], e[:-1]
    # the expected total equals n only up to the integration error: rescale to n
    e = e * (o.sum() / e.sum())
    stat = float(((o - e) ** 2 / e).sum())
    dof = len(o) - 1
    return float(stats.chi2.sf(stat, dof)), stat, dof, float(drawn.mean())


def albedo_two_ways(sample, eval_fp, mat, wo, n=1_000_000, seed=1):
    """Directional albedo (per channel) by importance sampling and by uniform sphere
    sampling, with their standard errors: ((mean_is, se_is), (mean_uni, se_uni))."""
    rng = np.random.default_rng(seed)
    mats, wos = _tile(mat, wo, n)
    out = sample(mats, wos, rng.random((n, 3)))
    drawn = out[:, 0] > 0
    wi = out[:, 4:7]
    wi_ok = np.where(drawn[:, None], wi, np.array([0.0, 0.0, 1.0]))
    ev = eval_fp(mats, wos, wi_ok)
    ev[:, 3] *= transmission_density_factor(mat, wo, wi_ok)
    cos = np.abs(wi[:, 2])
    with np.errstate(divide="ignore", invalid="ignore"):
        v_is = np.where(drawn[:, None] & (ev[:, 3:4] > 0), ev[:, 0:3] * cos[:, None] / ev[:, 3:4], 0.0)
    u = rng.random((n, 2))
    c = 1.0 - 2.0 * u[:, 0]
    s = np.sqrt(np.maximum(0.0, 1.0 - c * c))
    wu = np.stack([s * np.cos(TWO_PI * u[:, 1]), s * np.sin(TWO_PI * u[:, 1]), c], 1)
    ev2 = eval_fp(mats, wos, wu)
    v_un = ev2[:, 0:3] * np.abs(c)[:, None] * (4.0 * np.pi)
    se = lambda v: v.std(0) / np.sqrt(len(v))
    return (v_is.mean(0), se(v_is)), (v_un.mean(0), se(v_un)), v_is


# materials and outgoing directions of the checks: every lobe of the three aggregate
# materials, isotropic and anisotropic, front and (for transmission) back side
CASES = [
    ("diffuse", material("diffuse", color=0.8), 35.0),
    ("diffuse grazing", material("diffuse", color=0.8), 80.0),
    ("metal r0.3", material("metal", roughness=0.3), 35.0),
    ("metal r0.5 aniso0.7", material("metal", roughness=0.5, anisotropic=0.7), 60.0),
    ("disney diffuse+spec r0.5 clearcoat", material("disney", roughness=0.5, clearcoat=1.0,
                                                      clearcoat_gloss=0.0), 40.0),
    ("disney metallic r0.35", material("disney", metallic=1.0, roughness=0.35), 30.0),
    ("disney sheen aniso r0.6", material("disney", roughness=0.6, sheen=1.0, sheen_tint=0.5,
                                         anisotropic=0.6, specular_tint=0.5), 55.0),
    ("disney transmission r0.4", material("disney", roughness=0.4, transmission=0.9), 30.0),
    ("disney transmission back side", material("disney", roughness=0.5, transmission=0.8), 150.0),
]
