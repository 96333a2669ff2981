// Surface scattering for the wavefront shade stage. Each material follows the
// reference's local-space component and the BSDFAggregate wrapper around it:
//   aggregate / shading frame : builtin/btrc/builtin/material/utils/aggregate.cpp:32-229,
//                               builtin/btrc/builtin/material/utils/shader_frame.cpp:5-95
//   diffuse                   : builtin/btrc/builtin/material/component/diffuse.cpp:10-60
//   GGX conductor (metal)     : builtin/btrc/builtin/material/component/microfacet_reflection.h:10-121
//   Disney                    : builtin/btrc/builtin/material/disney.cpp:9-736
//   mirror / invisible / black: builtin/btrc/builtin/material/{mirror,invisible,black}.cpp
// Microfacet helpers: builtin/btrc/builtin/material/utils/microfacet.cpp:19-110,
// Fresnel: builtin/btrc/builtin/material/utils/fresnel.cpp:5-49.
#pragma once

#include "bmath.h"
#include "layout.h"

namespace bt {

struct CompSample
{
    V3 f;
    V3 dir;
    float pdf;
    bool is_delta;
};

BT_HD CompSample comp_clear()
{
    CompSample s;
    s.f = V3(0);
    s.dir = V3(0);
    s.pdf = 0;
    s.is_delta = false;
    return s;
}

BT_HD float sqrf(float x) { return x * x; }

// ---------------------------------------------------------------- distributions

BT_HD V3 sample_hemisphere_zweighted(float u1, float u2)
{
    float sx = 0, sy = 0;
    u1 = 2.0f * u1 - 1.0f;
    u2 = 2.0f * u2 - 1.0f;
    if(u1 != 0.0f || u2 != 0.0f)
    {
        // theta in units of pi
        float theta, r;
        if(fabsf(u1) > fabsf(u2))
        {
            r = u1;
            theta = 0.25f * (u2 / u1);
        }
        else
        {
            r = u2;
            theta = 0.5f - 0.25f * (u1 / u2);
        }
        float st, ct;
        sincos_pi(theta, st, ct);
        sx = r * ct;
        sy = r * st;
    }
    const float z = sqrtf(fmaxf(0.0f, 1.0f - (sx * sx + sy * sy)));
    return V3(sx, sy, z);
}

BT_HD float pdf_hemisphere_zweighted(V3 v) { return v.z >= 0 ? v.z / PI : 0.0f; }

BT_HD V3 sample_sphere_uniform(float u1, float u2)
{
    const float z = 1.0f - (u1 + u1);
    const float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float sp, cp;
    sincos_pi(2.0f * u2, sp, cp);
    return V3(r * cp, r * sp, z);
}

// Numerics. The reference evaluates these quantities as sqrt(1 - c*c), sin/cos of
// atan2(y, x) and sqrt(1 - z*z) / z. The same quantities are computed here in forms that
// stay accurate in FP32 near the specular peak, where 1 - c*c cancels catastrophically
// and the microfacet distribution amplifies that error by ~1/alpha^2:
//   sqrt(1 - c^2)        -> sqrt((1 - c)(1 + c))   (1 - c is exact for c in [0.5, 1])
//   cos/sin(atan2(y, x)) -> x / r, y / r           (r = |(x, y)|; 1, 0 when r == 0)
//   sin(theta_h)         -> |(h.x, h.y)|           (h a normalised half vector)
// The values are mathematically identical; only the FP32 rounding differs.
BT_HD float cos2sin(float c) { return sqrtf(fmaxf(0.0f, (1.0f - c) * (1.0f + c))); }

BT_HD float tan_theta(V3 w)
{
    const float t = (1.0f - w.z) * (1.0f + w.z);
    return t > 0 ? sqrtf(t) / w.z : 0.0f;
}

// cos(phi), sin(phi) of the azimuth of w
BT_HD void phi_cs(V3 w, float &c, float &s)
{
    const float r2 = w.x * w.x + w.y * w.y;
    if(r2 > 0.0f)
    {
        const float inv = 1.0f / sqrtf(r2);
        c = w.x * inv;
        s = w.y * inv;
    }
    else
    {
        c = 1.0f;
        s = 0.0f;
    }
}

// sin(theta) of a normalised vector
BT_HD float sin_theta_n(V3 w) { return sqrtf(w.x * w.x + w.y * w.y); }

// anisotropic GTR2 D of a normalised half vector
BT_HD float gtr2_of(V3 h, float ax, float ay);

// ---------------------------------------------------------------- fresnel

BT_HD float dielectric_fresnel(float eta_i, float eta_o, float cos_theta_i)
{
    if(cos_theta_i < 0)
    {
        const float t = eta_i;
        eta_i = eta_o;
        eta_o = t;
        cos_theta_i = -cos_theta_i;
    }
    const float sin_theta_i = cos2sin(cos_theta_i);
    const float sin_theta_t = eta_o / eta_i * sin_theta_i;
    if(sin_theta_t >= 1)
        return 1.0f;
    const float cos_theta_t = cos2sin(sin_theta_t);
    const float para = (eta_i * cos_theta_i - eta_o * cos_theta_t) / (eta_i * cos_theta_i + eta_o * cos_theta_t);
    const float perp = (eta_o * cos_theta_i - eta_i * cos_theta_t) / (eta_o * cos_theta_i + eta_i * cos_theta_t);
    return 0.5f * (para * para + perp * perp);
}

BT_HD float schlick(float R0, float c)
{
    const float t = 1.0f - c, t2 = t * t;
    return R0 + (1.0f - R0) * (t2 * t2 * t);
}

BT_HD V3 schlick3(V3 R0, float c)
{
    const float t = 1.0f - c, t2 = t * t, t5 = t2 * t2 * t;
    return R0 + (V3(1.0f) - R0) * t5;
}

// ---------------------------------------------------------------- microfacet

BT_HD float mf_smith_gtr2(float tan_t, float alpha)
{
    if(tan_t == 0)
        return 1.0f;
    const float root = alpha * tan_t;
    return 2.0f / (1.0f + sqrtf(1.0f + root * root));
}

BT_HD float mf_aniso_gtr2(float sin_phi_h, float cos_phi_h, float sin_theta_h, float cos_theta_h, float ax, float ay)
{
    const float A = sqrf(cos_phi_h / ax) + sqrf(sin_phi_h / ay);
    const float RD = sqrf(sin_theta_h) * A + sqrf(cos_theta_h);
    return 1.0f / (PI * ax * ay * sqrf(RD));
}

BT_HD float gtr2_of(V3 h, float ax, float ay)
{
    float c, s;
    phi_cs(h, c, s);
    return mf_aniso_gtr2(s, c, sin_theta_n(h), h.z, ax, ay);
}

BT_HD float mf_smith_aniso_gtr2(float cos_phi, float sin_phi, float ax, float ay, float tan_t)
{
    const float t = sqrf(ax * cos_phi) + sqrf(ay * sin_phi);
    const float sq = 1.0f + t * sqrf(tan_t);
    const float lambda = -0.5f + 0.5f * sqrtf(sq);
    return 1.0f / (1.0f + lambda);
}

BT_HD V3 mf_sample_aniso_gtr2(float ax, float ay, float s0, float s1)
{
    float sp, cp;
    sincos_pi(2.0f * s0, sp, cp);
    float sin_phi_h = ay * sp;
    float cos_phi_h = ax * cp;
    const float nor = 1.0f / sqrtf(sqrf(sin_phi_h) + sqrf(cos_phi_h));
    sin_phi_h *= nor;
    cos_phi_h *= nor;
    const float A = sqrf(cos_phi_h / ax) + sqrf(sin_phi_h / ay);
    const float cos_theta_h = sqrtf(A * (1.0f - s1) / ((1.0f - A) * s1 + A));
    const float sin_theta_h = cos2sin(cos_theta_h);
    return normalize(V3(sin_theta_h * cos_phi_h, sin_theta_h * sin_phi_h, cos_theta_h));
}

BT_HD float mf_gtr1(float sin_theta_h, float cos_theta_h, float alpha)
{
    const float U = sqrf(alpha) - 1;
    const float LD = 2.0f * PI * logf(alpha);
    const float RD = sqrf(alpha * cos_theta_h) + sqrf(sin_theta_h);
    return U / (LD * RD);
}

BT_HD V3 mf_sample_gtr1(float alpha, float s0, float s1)
{
    const float cos_theta = sqrtf((powf(alpha, 2.0f - 2.0f * s1) - 1.0f) / (sqrf(alpha) - 1.0f));
    const float sin_theta = cos2sin(cos_theta);
    float sp, cp;
    sincos_pi(2.0f * s0, sp, cp);
    return normalize(V3(sin_theta * cp, sin_theta * sp, cos_theta));
}

BT_HD V3 mf_sample_vndf(V3 ve, float ax, float ay, float s0, float s1)
{
    const V3 vh = normalize(V3(ax * ve.x, ay * ve.y, ve.z));
    const float lensq = vh.x * vh.x + vh.y * vh.y;
    V3 t1(1, 0, 0);
    if(lensq > 3e-4f)
        t1 = V3(-vh.y, vh.x, 0) / sqrtf(lensq);
    const V3 t2 = cross(vh, t1);
    const float r = sqrtf(s0);
    float sp, cp;
    sincos_pi(2.0f * s1, sp, cp);
    const float tt1 = r * cp;
    const float tt2_ = r * sp;
    const float s = 0.5f * (1.0f + vh.z);
    const float tt2 = (1.0f - s) * sqrtf(1.0f - tt1 * tt1) + s * tt2_;
    const V3 nh = tt1 * t1 + tt2 * t2 + sqrtf(fmaxf(0.0f, 1.0f - tt1 * tt1 - tt2 * tt2)) * vh;
    return normalize(V3(ax * nh.x, ay * nh.y, fmaxf(0.0f, nh.z)));
}

// ---------------------------------------------------------------- diffuse component

BT_HD V3 diffuse_eval(V3 albedo, V3 lwi, V3 lwo)
{
    return (lwi.z <= 0 || lwo.z <= 0) ? V3(0) : albedo / PI;
}

BT_HD float diffuse_pdf(V3 lwi, V3 lwo)
{
    return (lwi.z <= 0 || lwo.z <= 0) ? 0.0f : pdf_hemisphere_zweighted(lwi);
}

// ---------------------------------------------------------------- GGX conductor component

struct MetalParams
{
    V3 R0;
    float ax, ay;
};

BT_HD MetalParams metal_params(const float *p)
{
    MetalParams m;
    m.R0 = V3(p[0], p[1], p[2]);
    const float roughness = p[3], aniso = p[4];
    float aspect = 1.0f;
    if(aniso > 0)
        aspect = sqrtf(1.0f - 0.9f * aniso);
    m.ax = fmaxf(0.001f, roughness * roughness / aspect);
    m.ay = fmaxf(0.001f, roughness * roughness * aspect);
    return m;
}

BT_HD void metal_eval_pdf(const MetalParams &m, V3 lwi, V3 lwo, V3 &f, float &pdf)
{
    if(lwi.z <= 0 || lwo.z <= 0)
    {
        f = V3(0);
        pdf = 0;
        return;
    }
    const float cti = lwi.z, cto = lwo.z;
    const V3 lwh = normalize(lwi + lwo);
    const float ctd = dot(lwi, lwh);
    const float D = gtr2_of(lwh, m.ax, m.ay);
    float cpi, spi, cpo, spo;
    phi_cs(lwi, cpi, spi);
    phi_cs(lwo, cpo, spo);
    const float Go = mf_smith_aniso_gtr2(cpo, spo, m.ax, m.ay, tan_theta(lwo));
    const float Gi = mf_smith_aniso_gtr2(cpi, spi, m.ax, m.ay, tan_theta(lwi));
    const V3 F = schlick3(m.R0, ctd);
    f = F * (D * Gi * Go / fabsf(4.0f * cti * cto));
    pdf = Go * D / (4.0f * lwo.z);
}

// ---------------------------------------------------------------- Disney component

struct DisneyParams
{
    V3 C, C_tint;
    float metallic, roughness, specular, specular_tint, anisotropic, sheen, sheen_tint;
    float clearcoat, clearcoat_roughness, transmission, transmission_roughness, ior;
    float trans_ax, trans_ay, ax, ay;
    float w_diffuse, w_specular, w_clearcoat, w_transmission;
};

BT_HD float one_minus_5(float x)
{
    const float t = 1.0f - x, t2 = t * t;
    return t2 * t2 * t;
}

BT_HD DisneyParams disney_params(const float *p)
{
    DisneyParams d;
    d.C = V3(p[0], p[1], p[2]);
    const float lum = luminance(d.C);
    d.C_tint = lum > 0 ? d.C / lum : V3(1.0f);
    d.metallic = p[3];
    d.roughness = p[4];
    d.specular = p[5];
    d.specular_tint = p[6];
    d.anisotropic = p[7];
    d.sheen = p[8];
    d.sheen_tint = p[9];
    d.clearcoat = p[10];
    const float clearcoat_gloss = p[11];
    d.transmission = p[12];
    d.transmission_roughness = p[13];
    d.ior = fmaxf(1.01f, p[14]);
    float aspect = 1.0f;
    if(d.anisotropic > 0)
        aspect = sqrtf(1.0f - 0.9f * d.anisotropic);
    d.ax = fmaxf(0.001f, sqrf(d.roughness) / aspect);
    d.ay = fmaxf(0.001f, sqrf(d.roughness) * aspect);
    d.trans_ax = fmaxf(0.001f, sqrf(d.transmission_roughness) / aspect);
    d.trans_ay = fmaxf(0.001f, sqrf(d.transmission_roughness) * aspect);
    d.clearcoat_roughness = fmaxf(0.0001f, sqrf(lerpf(0.1f, 0.0f, clearcoat_gloss)));
    const float A = clampf(lum * (1.0f - d.metallic), 0.3f, 0.7f);
    const float B = 1.0f - A;
    d.w_diffuse = A * (1.0f - d.transmission);
    d.w_transmission = A * d.transmission;
    d.w_specular = B * 2.0f / (2.0f + d.clearcoat);
    d.w_clearcoat = B * d.clearcoat / (2.0f + d.clearcoat);
    return d;
}

BT_HD bool disney_refract(V3 w, V3 n, float eta, V3 &out)
{
    const float cti = dot(w, n);
    const float s2t = sqrf(eta) * (1.0f - sqrf(cti));
    const float c2t = 1.0f - s2t;
    if(c2t <= 0)
        return false;
    const float ctt = sqrtf(c2t);
    out = normalize((eta * cti - ctt) * n - eta * w);
    return true;
}

BT_HD V3 disney_eval_trans(const DisneyParams &d, V3 lwi, V3 lwo)
{
    const float cti = lwi.z, cto = lwo.z;
    const float eta = cto > 0 ? d.ior : 1.0f / d.ior;
    V3 lwh = normalize(lwo + eta * lwi);
    if(lwh.z < 0)
        lwh = -lwh;
    const float ctd = dot(lwo, lwh);
    const float F = dielectric_fresnel(d.ior, 1, ctd);
    const float D = gtr2_of(lwh, d.trans_ax, d.trans_ay);
    float cpi, spi, cpo, spo;
    phi_cs(lwi, cpi, spi);
    phi_cs(lwo, cpo, spo);
    const float G = mf_smith_aniso_gtr2(cpi, spi, d.trans_ax, d.trans_ay, tan_theta(lwi)) *
                    mf_smith_aniso_gtr2(cpo, spo, d.trans_ax, d.trans_ay, tan_theta(lwo));
    const float sdem = ctd + eta * dot(lwi, lwh);
    const float corr = 1.0f / eta;  // radiance transport
    const V3 sqrtC(sqrtf(d.C.x), sqrtf(d.C.y), sqrtf(d.C.z));
    const float val = (1.0f - F) * D * G * eta * eta * dot(lwi, lwh) * dot(lwo, lwh) * corr * corr /
                      (cti * cto * sdem * sdem);
    const float trans_factor = cto > 0 ? d.transmission : 1.0f;
    return sqrtC * ((1.0f - d.metallic) * trans_factor * fabsf(val));
}

BT_HD V3 disney_eval_inner_refl(const DisneyParams &d, V3 lwi, V3 lwo)
{
    const V3 lwh = -normalize(lwi + lwo);
    const float ctd = dot(lwo, lwh);
    const float F = dielectric_fresnel(d.ior, 1, ctd);
    const float D = gtr2_of(lwh, d.trans_ax, d.trans_ay);
    float cpi, spi, cpo, spo;
    phi_cs(lwi, cpi, spi);
    phi_cs(lwo, cpo, spo);
    const float G = mf_smith_aniso_gtr2(cpi, spi, d.trans_ax, d.trans_ay, tan_theta(lwi)) *
                    mf_smith_aniso_gtr2(cpo, spo, d.trans_ax, d.trans_ay, tan_theta(lwo));
    return d.C * (d.transmission * fabsf(F * D * G / (4.0f * lwi.z * lwo.z)));
}

BT_HD V3 disney_eval_specular(const DisneyParams &d, V3 lwi, V3 lwo)
{
    const float cti = lwi.z, cto = lwo.z;
    const V3 lwh = normalize(lwi + lwo);
    const float ctd = dot(lwi, lwh);
    const V3 Cspec = lerp3(lerp3(V3(1.0f), d.C_tint, d.specular_tint), d.C, d.metallic);
    const V3 dielectric = Cspec * dielectric_fresnel(d.ior, 1.0f, ctd);
    const V3 conductor = schlick3(Cspec, ctd);
    const V3 F = lerp3(d.specular * dielectric, conductor, d.metallic);
    const float D = gtr2_of(lwh, d.ax, d.ay);
    float cpi, spi, cpo, spo;
    phi_cs(lwi, cpi, spi);
    phi_cs(lwo, cpo, spo);
    const float G = mf_smith_aniso_gtr2(cpi, spi, d.ax, d.ay, tan_theta(lwi)) *
                    mf_smith_aniso_gtr2(cpo, spo, d.ax, d.ay, tan_theta(lwo));
    return F * (D * G / fabsf(4.0f * cti * cto));
}

BT_HD V3 disney_eval(const DisneyParams &d, V3 lwi, V3 lwo)
{
    if(fabsf(lwi.z) < 1e-4f || fabsf(lwo.z) < 1e-4f)
        return V3(0);
    if(lwi.z * lwo.z < 0)
        return d.transmission == 0.0f ? V3(0) : disney_eval_trans(d, lwi, lwo);
    if(lwi.z < 0 && lwo.z < 0)
        return d.transmission == 0.0f ? V3(0) : disney_eval_inner_refl(d, lwi, lwo);
    if(lwi.z <= 0 || lwo.z <= 0)
        return V3(0);
    const float cti = lwi.z, cto = lwo.z;
    const V3 lwh = normalize(lwi + lwo);
    const float ctd = dot(lwi, lwh);
    V3 diffuse(0), sheen(0);
    if(d.metallic < 1.0f)
    {
        const V3 lambert = d.C / PI;
        const float fl = one_minus_5(cti), fv = one_minus_5(cto);
        const float rr = 2.0f * d.roughness * ctd * ctd;
        const V3 retro = d.C / PI * (rr * (fl + fv + fl * fv * (rr - 1)));
        diffuse = lambert * ((1.0f - 0.5f * fl) * (1.0f - 0.5f * fv)) + retro;
        if(d.sheen > 0.0f)
            sheen = 4.0f * d.sheen * lerp3(V3(1.0f), d.C_tint, d.sheen_tint) * one_minus_5(ctd);
    }
    const V3 specular = disney_eval_specular(d, lwi, lwo);
    V3 clearcoat(0);
    if(d.clearcoat > 0.0f)
    {
        const float tti = tan_theta(lwi), tto = tan_theta(lwo);
        const float cth = lwh.z, sth = sin_theta_n(lwh);
        const float D = mf_gtr1(sth, cth, d.clearcoat_roughness);
        const float F = schlick(0.04f, ctd);
        const float G = mf_smith_gtr2(tti, 0.25f) * mf_smith_gtr2(tto, 0.25f);
        const float val = d.clearcoat * D * F * G / fabsf(4.0f * cti * cto);
        clearcoat = V3(val);
    }
    return (diffuse + sheen) * ((1.0f - d.metallic) * (1.0f - d.transmission)) + specular + clearcoat;
}

BT_HD float disney_pdf_transmission(const DisneyParams &d, V3 lwi, V3 lwo)
{
    const float eta = lwo.z > 0 ? d.ior : 1.0f / d.ior;
    V3 lwh = normalize(lwo + eta * lwi);
    if(lwh.z < 0)
        lwh = -lwh;
    if(((lwo.z > 0) != (dot(lwh, lwo) > 0)) || ((lwi.z > 0) != (dot(lwh, lwi) > 0)))
        return 0.0f;
    const float sdem = dot(lwo, lwh) + eta * dot(lwi, lwh);
    const float dwh_to_dwi = eta * eta * dot(lwi, lwh) / (sdem * sdem);
    const float D = gtr2_of(lwh, d.trans_ax, d.trans_ay);
    return fabsf(dot(lwi, lwh) * D * dwh_to_dwi);
}

BT_HD float disney_pdf_inner_refl(const DisneyParams &d, V3 lwi, V3 lwo)
{
    const V3 lwh = -normalize(lwi + lwo);
    const float cth = lwh.z;
    const float ctd = dot(lwi, lwh);
    const float D = gtr2_of(lwh, d.trans_ax, d.trans_ay);
    return fabsf(cth * D / (4.0f * ctd));
}

BT_HD float disney_pdf(const DisneyParams &d, V3 lwi, V3 lwo)
{
    if(fabsf(lwi.z) < 1e-4f || fabsf(lwo.z) < 1e-4f)
        return 0.0f;
    if(lwo.z < 0)
    {
        if(d.transmission == 0.0f)
            return 0.0f;
        const float macro_F = clampf(dielectric_fresnel(d.ior, 1, lwo.z), 0.1f, 0.9f);
        if(lwi.z > 0)
            return (1.0f - macro_F) * disney_pdf_transmission(d, lwi, lwo);
        return macro_F * disney_pdf_inner_refl(d, lwi, lwo);
    }
    if(lwi.z < 0)
        return d.w_transmission * disney_pdf_transmission(d, lwi, lwo);
    const float diffuse = pdf_hemisphere_zweighted(lwi);
    const V3 lwh = normalize(lwi + lwo);
    const float cth = lwh.z, sth = sin_theta_n(lwh);
    const float ctd = dot(lwi, lwh);
    // the reference derives sin(phi_o) as sqrt(1 - cos^2), i.e. always non-negative
    float cpo, spo;
    phi_cs(lwo, cpo, spo);
    spo = fabsf(spo);
    const float spec_D = gtr2_of(lwh, d.ax, d.ay);
    const float pdf_spec = mf_smith_aniso_gtr2(cpo, spo, d.ax, d.ay, tan_theta(lwo)) * spec_D / (4.0f * lwo.z);
    const float cc_D = mf_gtr1(sth, cth, d.clearcoat_roughness);
    const float pdf_cc = cth * cc_D / (4.0f * ctd);
    return d.w_diffuse * diffuse + d.w_specular * pdf_spec + d.w_clearcoat * pdf_cc;
}

// disney_eval and disney_pdf in one pass: in the reflection case (both directions above
// the surface) the half vector, the specular D, the outgoing Smith G, both tangents and
// the clearcoat D are shared, each computed by the same expression as in the separate
// functions; the other cases call them.
BT_HD void disney_eval_pdf_split(const DisneyParams &d, V3 lwi, V3 lwo, V3 &f, float &pdf)
{
    f = disney_eval(d, lwi, lwo);
    pdf = disney_pdf(d, lwi, lwo);
}

BT_HD void disney_eval_pdf(const DisneyParams &d, V3 lwi, V3 lwo, V3 &f, float &pdf)
{
    if(!(lwi.z >= 1e-4f && lwo.z >= 1e-4f))
    {
        disney_eval_pdf_split(d, lwi, lwo, f, pdf);
        return;
    }
    const float cti = lwi.z, cto = lwo.z;
    const V3 lwh = normalize(lwi + lwo);
    const float ctd = dot(lwi, lwh);
    const float cth = lwh.z, sth = sin_theta_n(lwh);
    const float tti = tan_theta(lwi), tto = tan_theta(lwo);
    V3 diffuse(0), sheen(0);
    if(d.metallic < 1.0f)
    {
        const V3 lambert = d.C / PI;
        const float fl = one_minus_5(cti), fv = one_minus_5(cto);
        const float rr = 2.0f * d.roughness * ctd * ctd;
        const V3 retro = d.C / PI * (rr * (fl + fv + fl * fv * (rr - 1)));
        diffuse = lambert * ((1.0f - 0.5f * fl) * (1.0f - 0.5f * fv)) + retro;
        if(d.sheen > 0.0f)
            sheen = 4.0f * d.sheen * lerp3(V3(1.0f), d.C_tint, d.sheen_tint) * one_minus_5(ctd);
    }
    // specular (disney_eval_specular)
    const V3 Cspec = lerp3(lerp3(V3(1.0f), d.C_tint, d.specular_tint), d.C, d.metallic);
    const V3 dielectric = Cspec * dielectric_fresnel(d.ior, 1.0f, ctd);
    const V3 conductor = schlick3(Cspec, ctd);
    const V3 Fs = lerp3(d.specular * dielectric, conductor, d.metallic);
    const float Ds = gtr2_of(lwh, d.ax, d.ay);
    float cpi, spi, cpo, spo;
    phi_cs(lwi, cpi, spi);
    phi_cs(lwo, cpo, spo);
    // G is even in sin(phi): the pdf's |sin(phi_o)| gives the same Go
    const float Go = mf_smith_aniso_gtr2(cpo, spo, d.ax, d.ay, tto);
    const float G = mf_smith_aniso_gtr2(cpi, spi, d.ax, d.ay, tti) * Go;
    const V3 specular = Fs * (Ds * G / fabsf(4.0f * cti * cto));
    const float cc_D = mf_gtr1(sth, cth, d.clearcoat_roughness);
    V3 clearcoat(0);
    if(d.clearcoat > 0.0f)
    {
        const float Fc = schlick(0.04f, ctd);
        const float Gc = mf_smith_gtr2(tti, 0.25f) * mf_smith_gtr2(tto, 0.25f);
        clearcoat = V3(d.clearcoat * cc_D * Fc * Gc / fabsf(4.0f * cti * cto));
    }
    f = (diffuse + sheen) * ((1.0f - d.metallic) * (1.0f - d.transmission)) + specular + clearcoat;
    const float pdf_spec = Go * Ds / (4.0f * lwo.z);
    const float pdf_cc = cth * cc_D / (4.0f * ctd);
    pdf = d.w_diffuse * pdf_hemisphere_zweighted(lwi) + d.w_specular * pdf_spec + d.w_clearcoat * pdf_cc;
}

BT_HD V3 disney_sample_transmission(const DisneyParams &d, V3 lwo, float s0, float s1)
{
    const V3 lwh = mf_sample_aniso_gtr2(d.trans_ax, d.trans_ay, s0, s1);
    if(lwh.z <= 0)
        return V3(0);
    if((lwo.z > 0) != (dot(lwh, lwo) > 0))
        return V3(0);
    const float eta = lwo.z > 0 ? 1.0f / d.ior : d.ior;
    const V3 owh = dot(lwh, lwo) > 0 ? lwh : -lwh;
    V3 lwi;
    if(!disney_refract(lwo, owh, eta, lwi))
        return V3(0);
    if(lwi.z * lwo.z > 0 || ((lwi.z > 0) != (dot(lwh, lwi) > 0)))
        return V3(0);
    return normalize(lwi);
}

BT_HD V3 disney_sample_inner_refl(const DisneyParams &d, V3 lwo, float s0, float s1)
{
    const V3 lwh = mf_sample_aniso_gtr2(d.trans_ax, d.trans_ay, s0, s1);
    if(lwh.z <= 0)
        return V3(0);
    const V3 lwi = 2.0f * dot(lwo, lwh) * lwh - lwo;
    if(lwi.z > 0)
        return V3(0);
    return normalize(lwi);
}

BT_HD V3 disney_sample_specular(const DisneyParams &d, V3 lwo, float s0, float s1)
{
    const V3 lwh = mf_sample_vndf(lwo, d.ax, d.ay, s0, s1);
    if(lwh.z <= 0)
        return V3(0);
    const V3 lwi = 2.0f * dot(lwo, lwh) * lwh - lwo;
    if(lwi.z <= 0)
        return V3(0);
    return normalize(lwi);
}

BT_HD V3 disney_sample_clearcoat(const DisneyParams &d, V3 lwo, float s0, float s1)
{
    const V3 lwh = mf_sample_gtr1(d.clearcoat_roughness, s0, s1);
    if(lwh.z <= 0)
        return V3(0);
    const V3 lwi = 2.0f * dot(lwo, lwh) * lwh - lwo;
    if(lwi.z <= 0)
        return V3(0);
    return normalize(lwi);
}

// Disney::sample direction (disney.cpp): lobe selection by s0, the lobe's sampler on
// (s1, s2); false when no direction results
BT_HD bool disney_sample_dir(const DisneyParams &d, V3 lwo, float s0, float s1, float s2, V3 &lwi)
{
    if(fabsf(lwo.z) < 1e-4f)
        return false;
    if(lwo.z < 0)
    {
        if(d.transmission == 0.0f)
            return false;
        const float macro_F = clampf(dielectric_fresnel(d.ior, 1, lwo.z), 0.1f, 0.9f);
        lwi = s0 >= macro_F ? disney_sample_transmission(d, lwo, s1, s2) : disney_sample_inner_refl(d, lwo, s1, s2);
    }
    else
    {
        float sel = s0;
        if(sel < d.w_diffuse)
            lwi = sample_hemisphere_zweighted(s1, s2);
        else
        {
            sel -= d.w_diffuse;
            if(sel < d.w_transmission)
                lwi = disney_sample_transmission(d, lwo, s1, s2);
            else
            {
                sel -= d.w_transmission;
                if(sel < d.w_specular)
                    lwi = disney_sample_specular(d, lwo, s1, s2);
                else
                    lwi = disney_sample_clearcoat(d, lwo, s1, s2);
            }
        }
    }
    return !(lwi.x == 0 && lwi.y == 0 && lwi.z == 0);
}

// handle_bad_sample (disney.cpp:566-573): a sample whose f |cos| / pdf exceeds 10 is dropped
BT_HD bool disney_bad_sample(V3 f, V3 lwi, float pdf)
{
    const V3 v = f * (fabsf(lwi.z) / pdf);
    return fmaxf(fmaxf(v.x, v.y), v.z) > 10;
}

// ---------------------------------------------------------------- shading frame + aggregate

struct ShaderFrame
{
    Frame geometry;
    Frame shading;

    BT_HD bool is_black_fringes(V3 w) const
    {
        return geometry.in_positive_z_hemisphere(w) != shading.in_positive_z_hemisphere(w);
    }
    BT_HD ShaderFrame flip_for_black_fringes(V3 wo) const
    {
        ShaderFrame f;
        f.geometry = geometry;
        f.shading = is_black_fringes(wo) ? geometry : shading;
        return f;
    }
    BT_HD float correct_shading_energy(V3 wi) const
    {
        const float down = fabsf(dot(geometry.z, wi));
        if(down > 1e-4f)
            return fabsf(dot(shading.z, wi)) / down;
        return 1.0f;
    }
    BT_HD float shadow_terminator(V3 wi) const
    {
        const float wgwi = dot(geometry.z, wi);
        const float wswi = dot(shading.z, wi);
        const float wgws = dot(geometry.z, shading.z);
        const float g = saturate(wgwi / (wswi * wgws));
        return -g * g * g + g * g + g;
    }
};

// Local-space component dispatch for the aggregate materials (diffuse, metal, disney).
struct MaterialEval
{
    int type;
    V3 albedo;           // diffuse / mirror / glass colour
    float glass_ior;
    MetalParams metal;
    DisneyParams disney;
};

BT_HD MaterialEval make_material_eval(const Material &m)
{
    MaterialEval e;
    e.type = m.type;
    e.albedo = V3(m.p[0], m.p[1], m.p[2]);
    e.glass_ior = m.p[3];
    if(m.type == MAT_METAL)
        e.metal = metal_params(m.p);
    else if(m.type == MAT_DISNEY)
        e.disney = disney_params(m.p);
    return e;
}

// Direction of the component's sample (diffuse: cosine hemisphere; metal: visible-normal
// GGX; disney: lobe selection); false when there is none.
BT_HD bool comp_sample_dir(const MaterialEval &e, V3 lwo, float s0, float s1, float s2, V3 &lwi)
{
    if(e.type == MAT_DIFFUSE)
    {
        if(lwo.z <= 0)
            return false;
        lwi = sample_hemisphere_zweighted(s1, s2);
        return true;
    }
    if(e.type == MAT_METAL)
    {
        if(lwo.z <= 0)
            return false;
        const V3 lwh = normalize(mf_sample_vndf(lwo, e.metal.ax, e.metal.ay, s1, s2));
        if(lwh.z <= 0)
            return false;
        lwi = normalize(2.0f * dot(lwo, lwh) * lwh - lwo);
        return lwi.z > 0;
    }
    return disney_sample_dir(e.disney, lwo, s0, s1, s2, lwi);
}

BT_HD void comp_eval_pdf(const MaterialEval &e, V3 lwi, V3 lwo, V3 &f, float &pdf)
{
    if(e.type == MAT_DIFFUSE)
    {
        f = diffuse_eval(e.albedo, lwi, lwo);
        pdf = diffuse_pdf(lwi, lwo);
    }
    else if(e.type == MAT_METAL)
        metal_eval_pdf(e.metal, lwi, lwo, f, pdf);
    else
        disney_eval_pdf(e.disney, lwi, lwo, f, pdf);
}

// a sampled direction with its f and pdf; Disney drops bad samples
BT_HD CompSample comp_finish(const MaterialEval &e, V3 lwi, V3 f, float pdf)
{
    if(e.type == MAT_DISNEY && disney_bad_sample(f, lwi, pdf))
        return comp_clear();
    CompSample r;
    r.dir = lwi;
    r.f = f;
    r.pdf = pdf;
    r.is_delta = false;
    return r;
}

BT_HD CompSample comp_sample(const MaterialEval &e, V3 lwo, float s0, float s1, float s2)
{
    V3 lwi;
    if(!comp_sample_dir(e, lwo, s0, s1, s2, lwi))
        return comp_clear();
    V3 f;
    float pdf;
    comp_eval_pdf(e, lwi, lwo, f, pdf);
    return comp_finish(e, lwi, f, pdf);
}

// Full surface shader: aggregate materials go through the shading-frame logic with a
// single component of weight 1; mirror / invisible / black are their own shaders.
struct SurfaceShader
{
    ShaderFrame frame;
    MaterialEval mat;
    bool shadow_terminator;

    BT_HD CompSample sample(V3 wo, float s0, float s1, float s2) const
    {
        V3 f;
        float pdf;
        return sample_eval(wo, s0, s1, s2, false, V3(0, 0, 1), f, pdf);
    }

    // BSDF sample for the path's next direction and, when want_li, f and pdf of the light
    // sample's direction wi_li (zero for delta shaders); the values are those of sample
    // and eval_pdf, each evaluation computing f and pdf in one pass.
    BT_HD CompSample sample_eval(V3 wo, float s0, float s1, float s2, bool want_li, V3 wi_li, V3 &f_li,
                                 float &pdf_li) const
    {
        f_li = V3(0);
        pdf_li = 0.0f;
        CompSample r = comp_clear();
        if(mat.type == MAT_BLACK)
            return r;
        if(mat.type == MAT_INVISIBLE)
        {
            r.f = V3(1.0f / fabsf(dot(frame.geometry.z, normalize(wo))));
            r.dir = -wo;
            r.pdf = 1;
            r.is_delta = true;
            return r;
        }
        const ShaderFrame fr = frame.flip_for_black_fringes(wo);
        if(mat.type == MAT_GLASS)
            return glass_sample(fr, wo, s0);
        if(mat.type == MAT_MIRROR)
        {
            V3 lwo = fr.shading.global_to_local(wo);
            if(lwo.z > 0)
            {
                lwo = normalize(lwo);
                const V3 wi = fr.shading.local_to_global(V3(-lwo.x, -lwo.y, lwo.z));
                if(!frame.is_black_fringes(wi))
                {
                    r.f = schlick3(mat.albedo, lwo.z) / lwo.z * fr.correct_shading_energy(wi);
                    r.dir = wi;
                    r.pdf = 1;
                    r.is_delta = true;
                }
            }
            return r;
        }
        const V3 lwo = normalize(fr.shading.global_to_local(wo));
        V3 lwi_bs(0, 0, 1);
        const bool has_bs = comp_sample_dir(mat, lwo, s0, s1, s2, lwi_bs);
        const V3 lwi_li = want_li ? normalize(fr.shading.global_to_local(wi_li)) : V3(0, 0, 1);
        V3 f_bs(0);
        float pdf_bs = 0.0f;
        if(has_bs)
            comp_eval_pdf(mat, lwi_bs, lwo, f_bs, pdf_bs);
        if(want_li)
        {
            comp_eval_pdf(mat, lwi_li, lwo, f_li, pdf_li);
            float kk = fr.correct_shading_energy(wi_li);
            if(shadow_terminator)
                kk *= frame.shadow_terminator(wi_li);
            f_li = f_li * kk;
        }
        if(!has_bs)
            return r;
        const CompSample c = comp_finish(mat, lwi_bs, f_bs, pdf_bs);
        if(c.pdf <= 0)
            return r;
        r.dir = fr.shading.local_to_global(c.dir);
        if(frame.is_black_fringes(r.dir))
            return comp_clear();
        r.pdf = c.pdf;
        float k = fr.correct_shading_energy(r.dir);
        if(shadow_terminator)
            k *= frame.shadow_terminator(r.dir);
        r.f = c.f * k;
        r.is_delta = false;
        return r;
    }

    // GlassShaderImpl::sample_bidir (builtin/btrc/builtin/material/glass.cpp:34-95): delta
    // reflection with probability F, else delta refraction; the refraction branch reports
    // pdf = 1 - F(cos of the refracted direction), as the reference does
    BT_HD CompSample glass_sample(const ShaderFrame &fr, V3 wo, float s0) const
    {
        CompSample r = comp_clear();
        const V3 color = mat.albedo;
        const float ior = mat.glass_ior;
        const V3 nwo = normalize(fr.shading.global_to_local(wo));
        const float F = dielectric_fresnel(ior, 1, nwo.z);
        if(s0 < F)
        {
            const V3 lwi(-nwo.x, -nwo.y, nwo.z);
            const V3 wi = fr.shading.local_to_global(lwi);
            if(frame.is_black_fringes(wi))
                return r;
            r.f = color * (F / fabsf(lwi.z)) * fr.correct_shading_energy(wi);
            r.dir = wi;
            r.pdf = F;
            r.is_delta = true;
            return r;
        }
        const float nz = nwo.z > 0 ? 1.0f : -1.0f;
        const float eta = nwo.z > 0 ? 1.0f / ior : ior;
        const float cti = fabsf(nwo.z);
        const float s2i = fmaxf(0.0f, 1.0f - cti * cti);
        const float s2t = eta * eta * s2i;
        if(s2t >= 1)
            return r;
        const float ctt = sqrtf(1.0f - s2t);
        const V3 nwi = normalize((eta * cti - ctt) * V3(0, 0, nz) - eta * nwo);
        const V3 wi = fr.shading.local_to_global(nwi);
        if(frame.is_black_fringes(wi))
            return r;
        const float corr = eta * eta;  // radiance transport
        r.f = color * (corr * (1.0f - F) / fabsf(nwi.z)) * fr.correct_shading_energy(wi);
        r.dir = wi;
        r.pdf = 1.0f - dielectric_fresnel(ior, 1, nwi.z);
        r.is_delta = true;
        return r;
    }

    BT_HD void eval_pdf(V3 wi, V3 wo, V3 &f, float &pdf) const
    {
        f = V3(0);
        pdf = 0.0f;
        if(mat.type == MAT_BLACK || mat.type == MAT_INVISIBLE || mat.type == MAT_MIRROR || mat.type == MAT_GLASS)
            return;
        const ShaderFrame fr = frame.flip_for_black_fringes(wo);
        const V3 lwi = normalize(fr.shading.global_to_local(wi));
        const V3 lwo = normalize(fr.shading.global_to_local(wo));
        float k = fr.correct_shading_energy(wi);
        if(shadow_terminator)
            k *= frame.shadow_terminator(wi);
        comp_eval_pdf(mat, lwi, lwo, f, pdf);
        f = f * k;
    }
};

} // namespace bt
