// Wavefront path tracer: per-bounce stage kernels over SoA path queues.
// Stage order per bounce follows WavefrontPathTracer::render
// (builtin/btrc/builtin/renderer/wavefront.cpp:205-325): generate -> trace -> [medium]
// -> shade -> shadow. Differences that are GB300-specific:
//   * queue counters stay in device memory; a one-thread control kernel advances them,
//     so there is no blocking device-to-host copy per bounce (the reference reads the
//     counters back every bounce, wavefront.cpp:284);
//   * the queue is topped up with new camera paths every bounce (the reference refills
//     only when half empty, generate.cpp:148-156); the estimator is unchanged;
//   * queue appends are warp-aggregated (one atomic per warp instead of per thread);
//   * two bounces (ping and pong buffers) are captured into one CUDA graph and relaunched.
#include <algorithm>
#include <cstdio>
#include <mutex>
#include <vector>

#include "bsdf.cuh"
#include "kernels.h"
#include "nrc.h"
#include "texture.h"
#include "traverse.cuh"
#include "two_level.cuh"

namespace bt {

__constant__ uint32_t c_primes[PRIME_COUNT];
// per Halton dimension: ceil(2^64 / prime) for exact division by a multiply, and the
// dimension's scrambling seed mix_bits(1 + (dim << 4))
__constant__ uint64_t c_prime_magic[PRIME_COUNT];
__constant__ uint64_t c_dim_hash[PRIME_COUNT];

namespace {

constexpr int BLOCK = 256;
constexpr uint32_t MAX_TRACKING_STEPS = 1u << 20;

// ---------------------------------------------------------------- small helpers

__device__ __forceinline__ V3 v3(const F4 &f) { return V3(f.x, f.y, f.z); }
__device__ __forceinline__ F4 f4(V3 v, float w) { return F4{ v.x, v.y, v.z, w }; }
__device__ __forceinline__ F4 ldf4(const F4 *p) { const float4 v = __ldg(reinterpret_cast<const float4 *>(p)); return F4{ v.x, v.y, v.z, v.w }; }

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// warp-aggregated queue append: one atomic per converged group of callers
__device__ __forceinline__ uint32_t queue_append(uint32_t *counter)
{
    const uint32_t mask = __activemask();
    const uint32_t leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if(lane_id() == leader)
        base = atomicAdd(counter, static_cast<uint32_t>(__popc(mask)));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(mask & ((1u << lane_id()) - 1u));
}

// Film::splat_atomic (core/btrc/core/film.cpp:131-165): non-finite values are dropped
__device__ __forceinline__ void splat(float4 *film, uint32_t pixel, int width, V3 v)
{
    if(!all_finite(v))
        return;
    const uint32_t x = pixel & 0xffffu, y = pixel >> 16;
    atomicAdd(film + (static_cast<size_t>(y) * width + x), make_float4(v.x, v.y, v.z, 0.0f));
}

// intersection_offset (common/btrc/utils/intersection.cpp:5-37)
__device__ __forceinline__ V3 offset_point(V3 pos, V3 nor)
{
    const float ORIGIN = 1.0f / 32.0f, FLOAT_SCALE = 1.0f / 65536.0f, INT_SCALE = 256.0f;
    const int ox = static_cast<int>(2 * INT_SCALE * nor.x);
    const int oy = static_cast<int>(2 * INT_SCALE * nor.y);
    const int oz = static_cast<int>(2 * INT_SCALE * nor.z);
    const float px = __int_as_float(__float_as_int(pos.x) + (pos.x < 0 ? -ox : ox));
    const float py = __int_as_float(__float_as_int(pos.y) + (pos.y < 0 ? -oy : oy));
    const float pz = __int_as_float(__float_as_int(pos.z) + (pos.z < 0 ? -oz : oz));
    return V3(fabsf(pos.x) < ORIGIN ? pos.x + FLOAT_SCALE * nor.x : px,
              fabsf(pos.y) < ORIGIN ? pos.y + FLOAT_SCALE * nor.y : py,
              fabsf(pos.z) < ORIGIN ? pos.z + FLOAT_SCALE * nor.z : pz);
}

__device__ __forceinline__ V3 offset_dir(V3 pos, V3 nor, V3 dir)
{
    return offset_point(pos, dot(nor, dir) > 0 ? nor : -nor);
}

__device__ __forceinline__ V3 aff_point(const float *m, V3 p)
{
    return V3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
              m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}
__device__ __forceinline__ V3 aff_vector(const float *m, V3 v)
{
    return V3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
              m[8] * v.x + m[9] * v.y + m[10] * v.z);
}
// normal transform from the inverse matrix (core ctransform.cpp apply_to_normal)
__device__ __forceinline__ V3 aff_normal(const float *inv, V3 n)
{
    return V3(inv[0] * n.x + inv[4] * n.y + inv[8] * n.z, inv[1] * n.x + inv[5] * n.y + inv[9] * n.z,
              inv[2] * n.x + inv[6] * n.y + inv[10] * n.z);
}

// ---------------------------------------------------------------- sampler

struct DSampler
{
    SamplerState s;
    int type;

    __device__ __forceinline__ float halton(uint32_t dim) const
    {
        return owen_scrambled_radical_inverse(c_primes[dim], s.a, c_dim_hash[dim], c_prime_magic[dim]);
    }
    __device__ __forceinline__ float get1d()
    {
        if(type == SAMPLER_INDEPENDENT)
            return pcg32_uniform(s.a, s.b);
        uint32_t dim = static_cast<uint32_t>(s.b);
        if(dim >= PRIME_COUNT)
            dim = 2;
        const float v = halton(dim);
        s.b = dim + 1;
        return v;
    }
    __device__ __forceinline__ void get2d(float &x, float &y)
    {
        if(type == SAMPLER_INDEPENDENT)
        {
            x = pcg32_uniform(s.a, s.b);
            y = pcg32_uniform(s.a, s.b);
            return;
        }
        uint32_t dim = static_cast<uint32_t>(s.b);
        if(dim + 1 >= PRIME_COUNT)
            dim = 2;
        x = halton(dim);
        y = halton(dim + 1);
        s.b = dim + 2;
    }
    __device__ __forceinline__ void get3d(float &x, float &y, float &z)
    {
        if(type == SAMPLER_INDEPENDENT)
        {
            x = pcg32_uniform(s.a, s.b);
            y = pcg32_uniform(s.a, s.b);
            z = pcg32_uniform(s.a, s.b);
            return;
        }
        uint32_t dim = static_cast<uint32_t>(s.b);
        if(dim + 2 >= PRIME_COUNT)
            dim = 2;
        x = halton(dim);
        y = halton(dim + 1);
        z = halton(dim + 2);
        s.b = dim + 3;
    }
};

__device__ __forceinline__ SamplerState sampler_init(int type, const HaltonConsts &hc, uint32_t px, uint32_t py,
                                                     uint32_t sample_index)
{
    SamplerState st;
    if(type == SAMPLER_INDEPENDENT)
    {
        pcg32_seed(st.a, st.b, murmur64a_2x32(px, py), PCG_STREAM);
        pcg32_advance(st.a, st.b, static_cast<uint64_t>(sample_index) * 65536u);
        return st;
    }
    uint64_t index = 0;
    if(hc.stride > 1)
    {
        const uint32_t pm[2] = { px % HALTON_MAX_RES, py % HALTON_MAX_RES };
        for(int i = 0; i < 2; ++i)
        {
            const uint64_t off = inverse_radical_inverse(pm[i], i == 0 ? 2u : 3u, hc.exponent[i]);
            index += off * static_cast<uint64_t>((hc.stride / hc.scale[i]) * hc.mult_inverse[i]);
        }
        index %= static_cast<uint64_t>(hc.stride);
    }
    index += static_cast<uint64_t>(sample_index) * static_cast<uint64_t>(hc.stride);
    st.a = index;
    st.b = 2;
    return st;
}

// ---------------------------------------------------------------- geometry helpers

struct SurfacePoint
{
    V3 position;
    Frame frame;
    V3 interp_z;
    float tu, tv;    // texture coordinate
};

// get_hitinfo (core/btrc/core/scene.cpp:9-64)
__device__ SurfacePoint get_hitinfo(const DevScene &S, V3 o, V3 d, const Instance &inst, uint32_t idx, float t,
                                    float b1, float b2)
{
    SurfacePoint sp;
    sp.position = o + t * d;
    const F4 *rec = S.shade + static_cast<size_t>(idx) * SHADE_F4;
    const F4 gx = ldf4(rec + 0), gy = ldf4(rec + 1), gz = ldf4(rec + 2);
    const F4 sa = ldf4(rec + 3), sba = ldf4(rec + 4), sca = ldf4(rec + 5);
    Frame f(v3(gx), v3(gy), v3(gz));
    f.x = normalize(aff_vector(inst.l2w, f.x));
    f.y = normalize(aff_vector(inst.l2w, f.y));
    f.z = normalize(aff_normal(inst.w2l, f.z));
    sp.frame = f;
    const V3 in = v3(sa) + v3(sba) * b1 + v3(sca) * b2;
    sp.interp_z = normalize(aff_normal(inst.w2l, in));
    sp.tu = gx.w + gy.w * b1 + gz.w * b2;
    sp.tv = sa.w + sba.w * b1 + sca.w * b2;
    return sp;
}

// ---------------------------------------------------------------- lights

__device__ __forceinline__ uint32_t alias_sample(const AliasEntry8 *table, uint32_t n, float u)
{
    const float nu = static_cast<float>(n) * u;
    const uint32_t i = min(static_cast<uint32_t>(nu), n - 1);
    const float s = nu - static_cast<float>(i);
    const AliasEntry8 e = table[i];
    return s <= e.accept ? i : e.alias;
}

__device__ __forceinline__ TexTables tex_tables(const DevScene &S)
{
    return TexTables{ S.tex_images, S.tex_texels, S.tex_instr };
}

// IBL::eval_local (builtin/btrc/builtin/light/ibl.cpp:69-77): (phi / 2 pi, theta / pi)
__device__ __forceinline__ V3 ibl_eval_local(const DevScene &S, V3 d)
{
    float phi = 0.0f;
    if(d.x != 0.0f || d.y != 0.0f)
    {
        phi = atan2f(d.y, d.x);
        phi = phi < 0 ? phi + 2 * PI : phi;
    }
    const float theta = acosf(fminf(fmaxf(d.z, -1.0f), 1.0f));
    const float u = saturate(1 / (2 * PI) * phi);
    const float v = saturate(1 / PI * theta);
    return tex_eval(tex_tables(S), S.env.prog, u, v);
}

__device__ __forceinline__ V3 ibl_to_local(const EnvLight &env, V3 g)
{
    return V3(dot(g, V3(env.frame_x[0], env.frame_x[1], env.frame_x[2])),
              dot(g, V3(env.frame_y[0], env.frame_y[1], env.frame_y[2])), dot(g, V3(env.up[0], env.up[1], env.up[2])));
}

// EnvirLightSampler::pdf (builtin/btrc/builtin/light/env_sampler.cpp:165-187)
__device__ float ibl_pdf_local(const DevScene &S, V3 to_light)
{
    const V3 dir = normalize(to_light);
    const float theta = acosf(fminf(fmaxf(dir.z, -1.0f), 1.0f));
    float phi = 0.0f;
    if(dir.x != 0.0f || dir.y != 0.0f)
    {
        phi = atan2f(dir.y, dir.x);
        phi = phi < 0 ? phi + 2 * PI : phi;
    }
    const float u = phi / (2 * PI), v = theta / PI;
    const int w = S.env.lut_w, h = S.env.lut_h;
    const int tx = min(max(static_cast<int>(floorf(u * w)), 0), w - 1);
    const int ty = min(max(static_cast<int>(floorf(v * h)), 0), h - 1);
    const float tile_pdf = S.env_probs[ty * w + tx];
    const float u0 = static_cast<float>(tx) / w, u1 = static_cast<float>(tx + 1) / w;
    const float v0 = static_cast<float>(ty) / h, v1 = static_cast<float>(ty + 1) / h;
    const float c0 = cos_pi(v0), c1 = cos_pi(v1);
    return tile_pdf * (1.0f / fabsf(2 * PI * (u1 - u0) * (c1 - c0)));
}

__device__ __forceinline__ V3 env_le(const DevScene &S, V3 to_light)
{
    const EnvLight &env = S.env;
    if(env.type == ENV_IBL)
        return ibl_eval_local(S, normalize(ibl_to_local(env, to_light)));
    const V3 up(env.up[0], env.up[1], env.up[2]);
    const float c = dot(up, normalize(to_light));
    const float s = saturate(0.5f * (c + 1.0f));
    return V3(env.lower[0], env.lower[1], env.lower[2]) * (1.0f - s) + V3(env.upper[0], env.upper[1], env.upper[2]) * s;
}

// pdf_li of the environment light (solid angle): uniform sphere for gradient_sky
__device__ __forceinline__ float env_pdf(const DevScene &S, V3 to_light)
{
    if(S.env.type == ENV_IBL)
        return ibl_pdf_local(S, ibl_to_local(S.env, to_light));
    return 1.0f / (4.0f * PI);
}

struct LightSample
{
    bool success;
    V3 o, d;
    float t1, light_pdf;
    V3 li;
};

// IBL::sample_li_inline (ibl.cpp:31-42) over EnvirLightSampler::sample (env_sampler.cpp:137-163)
__device__ __forceinline__ void sample_ibl(const DevScene &S, V3 ref_pos, V3 ref_nor, bool offset_origin, float s0,
                                        float s1, float s2, float select_pdf, LightSample &r)
{
    const int w = S.env.lut_w, h = S.env.lut_h;
    const uint32_t tile = alias_sample(S.env_alias, static_cast<uint32_t>(w * h), s0);
    const int ty = static_cast<int>(tile) / w, tx = static_cast<int>(tile) % w;
    const float tile_pdf = S.env_probs[tile];
    const float u0 = static_cast<float>(tx) / w, u1 = static_cast<float>(tx + 1) / w;
    const float v0 = static_cast<float>(ty) / h, v1 = static_cast<float>(ty + 1) / h;
    float cv0 = cos_pi(v0), cv1 = cos_pi(v1);
    if(cv0 > cv1)
    {
        const float t = cv0;
        cv0 = cv1;
        cv1 = t;
    }
    const float cos_theta = cv0 + s2 * (cv1 - cv0);
    const float sin_theta = cos2sin(cos_theta);
    float sp, cp;
    sincos_pi(2.0f * (u0 + (u1 - u0) * s1), sp, cp);
    const V3 local(sin_theta * cp, sin_theta * sp, cos_theta);
    const float in_tile_pdf = 1.0f / (2 * PI * (u1 - u0) * (cv1 - cv0));
    const V3 dir = V3(S.env.frame_x[0], S.env.frame_x[1], S.env.frame_x[2]) * local.x +
                   V3(S.env.frame_y[0], S.env.frame_y[1], S.env.frame_y[2]) * local.y +
                   V3(S.env.up[0], S.env.up[1], S.env.up[2]) * local.z;
    r.o = offset_origin ? offset_dir(ref_pos, ref_nor, dir) : ref_pos;
    r.d = dir;
    r.t1 = MAX_FLOAT;
    r.li = ibl_eval_local(S, local);
    r.light_pdf = select_pdf * (tile_pdf * in_tile_pdf);
}

// sample_light_li_impl (builtin/.../wavefront/helper.cpp:9-61); offset_origin selects the
// surface form (origin offset along the normal) or the medium form (origin = ref_pos)
__device__ LightSample sample_light(const DevScene &S, V3 ref_pos, V3 ref_nor, bool offset_origin, DSampler &smp)
{
    LightSample r;
    float s0, s1, s2;
    smp.get3d(s0, s1, s2);
    const float sel = smp.get1d();
    r.success = false;
    if(S.num_lights == 0)
        return r;
    const int idx = min(static_cast<int>(sel * static_cast<float>(S.num_lights)), S.num_lights - 1);
    const float select_pdf = 1.0f / static_cast<float>(S.num_lights);
    if(idx < S.num_area_lights)
    {
        // MeshLight::sample_li_inline (builtin/btrc/builtin/light/mesh_light.cpp:31-58)
        const AreaLight L = S.area_lights[idx];
        const Geometry g = S.geometries[L.geometry];
        const Instance &inst = S.instances[L.instance];
        const uint32_t base = __float_as_uint(g.pad);
        const uint32_t prim = alias_sample(S.light_alias + base, g.tri_count, s0);
        const float tq = sqrtf(s1);
        const float u = 1.0f - tq, v = tq * s2;
        const F4 pa = ldf4(S.light_pos + (base + prim) * 3 + 0);
        const F4 pb = ldf4(S.light_pos + (base + prim) * 3 + 1);
        const F4 pc = ldf4(S.light_pos + (base + prim) * 3 + 2);
        const V3 a = v3(pa), ba = v3(pb), ca = v3(pc);
        const V3 pos = a + ba * u + ca * v;
        const V3 ez = normalize(V3(pa.w, pb.w, pc.w));
        const V3 spos = aff_point(inst.l2w, pos);
        const V3 snor = normalize(aff_normal(inst.w2l, ez));
        const V3 pos_to_ref = ref_pos - spos;
        const float dist2 = length_square(pos_to_ref);
        const float pdf_sa = 1.0f / (L.scale * L.scale) * (1.0f / g.total_area) * dist2 /
                             fabsf(dot(snor, normalize(pos_to_ref)));
        const V3 rad = dot(pos_to_ref, snor) > 0 ? V3(L.intensity[0], L.intensity[1], L.intensity[2]) : V3(0);
        const V3 diff = spos - ref_pos;
        const V3 dst = offset_dir(spos, snor, -diff);
        r.o = offset_origin ? offset_dir(ref_pos, ref_nor, diff) : ref_pos;
        r.d = dst - r.o;
        r.t1 = 1.0f;
        r.li = rad;
        r.light_pdf = select_pdf * pdf_sa;
    }
    else if(S.env.type == ENV_IBL)
        sample_ibl(S, ref_pos, ref_nor, offset_origin, s0, s1, s2, select_pdf, r);
    else
    {
        // GradientSky::sample_li_inline (builtin/btrc/builtin/light/gradient_sky.cpp:28-35)
        const V3 dir = sample_sphere_uniform(s0, s1);
        r.o = offset_origin ? offset_dir(ref_pos, ref_nor, dir) : ref_pos;
        r.d = dir;
        r.t1 = MAX_FLOAT;
        r.li = env_le(S, dir);
        r.light_pdf = select_pdf * (1.0f / (4.0f * PI));
    }
    r.success = true;
    return r;
}

// eval_miss_le (helper.cpp:144-172)
__device__ __forceinline__ V3 miss_le(const DevScene &S, V3 d, V3 beta_le, float bsdf_pdf)
{
    if(S.env.type == ENV_NONE)
        return V3(0);
    const V3 le = env_le(S, d);
    if(bsdf_pdf < 0)
        return beta_le * le / -bsdf_pdf;
    const float light_pdf = (1.0f / static_cast<float>(S.num_lights)) * env_pdf(S, d);
    return beta_le * le / (bsdf_pdf + light_pdf);
}

// handle_intersected_light (helper.cpp:174-207) with MeshLight::eval_le / pdf_li
__device__ __forceinline__ V3 hit_light_le(const DevScene &S, V3 o, V3 d, const SurfacePoint &sp, V3 beta_le,
                                           float bsdf_pdf, int light)
{
    if(light < 0)
        return V3(0);
    const AreaLight L = S.area_lights[light];
    const V3 le = dot(sp.frame.z, -d) >= 0 ? V3(L.intensity[0], L.intensity[1], L.intensity[2]) : V3(0);
    if(bsdf_pdf < 0)
        return beta_le * le / -bsdf_pdf;
    float pdf_li = 0;
    const V3 to_ref = o - sp.position;
    if(dot(sp.frame.z, to_ref) > 0)
    {
        const float total_area = S.geometries[L.geometry].total_area;
        const float dist2 = length_square(to_ref);
        const float dist3 = sqrtf(dist2) * dist2;
        pdf_li = 1.0f / (L.scale * L.scale) * (1.0f / total_area) * dist3 / fabsf(dot(sp.frame.z, to_ref));
    }
    const float light_pdf = (1.0f / static_cast<float>(S.num_lights)) * pdf_li;
    return beta_le * le / (bsdf_pdf + light_pdf);
}

// simple_russian_roulette (helper.cpp:67-97); returns true when the path ends
__device__ __forceinline__ bool russian_roulette(V3 &beta, int depth, DSampler &smp, const DevRender &R)
{
    if(depth < R.min_depth)
        return false;
    if(depth >= R.max_depth)
        return true;
    const float sam = smp.get1d();
    if(luminance(beta) < R.rr_threshold)
    {
        if(sam > R.rr_cont_prob)
            return true;
        beta = beta / R.rr_cont_prob;
    }
    return false;
}

// Seed of the PCG stream that a shadow ray's medium transmittance draws from: a hash of
// the path's sampler state at the start of the stage that emits the ray (the medium
// stage for a scattering event, the shade stage for a surface vertex) and of that stage.
// The stream is then a function of the path alone, not of its queue slot, so a CPU
// restatement that follows the same sampler streams draws the same transmittance.
constexpr uint64_t SHADOW_FROM_MEDIUM = 1, SHADOW_FROM_SURFACE = 2;

__device__ __forceinline__ uint64_t shadow_stream_seed(const SamplerState &s, uint64_t stage)
{
    return mix_bits(s.a ^ mix_bits(s.b + stage));
}

// ---------------------------------------------------------------- media

// software trilinear lookup of channel c of an nch-channel grid (x fastest), normalised
// coordinates, clamp addressing
__device__ __forceinline__ float grid_trilinear(const float *g, int rx, int ry, int rz, int nch, int c, V3 uvw)
{
    const float fx = uvw.x * rx - 0.5f, fy = uvw.y * ry - 0.5f, fz = uvw.z * rz - 0.5f;
    const float flx = floorf(fx), fly = floorf(fy), flz = floorf(fz);
    const float tx = fx - flx, ty = fy - fly, tz = fz - flz;
    const int x0 = static_cast<int>(flx), y0 = static_cast<int>(fly), z0 = static_cast<int>(flz);
    const int xa = min(max(x0, 0), rx - 1), xb = min(max(x0 + 1, 0), rx - 1);
    const int ya = min(max(y0, 0), ry - 1), yb = min(max(y0 + 1, 0), ry - 1);
    const int za = min(max(z0, 0), rz - 1), zb = min(max(z0 + 1, 0), rz - 1);
    g += c;
    const size_t sx = nch, sy = static_cast<size_t>(rx) * nch, sz = static_cast<size_t>(rx) * ry * nch;
    const float c000 = __ldg(g + za * sz + ya * sy + xa * sx), c100 = __ldg(g + za * sz + ya * sy + xb * sx);
    const float c010 = __ldg(g + za * sz + yb * sy + xa * sx), c110 = __ldg(g + za * sz + yb * sy + xb * sx);
    const float c001 = __ldg(g + zb * sz + ya * sy + xa * sx), c101 = __ldg(g + zb * sz + ya * sy + xb * sx);
    const float c011 = __ldg(g + zb * sz + yb * sy + xa * sx), c111 = __ldg(g + zb * sz + yb * sy + xb * sx);
    const float c00 = c000 + (c100 - c000) * tx, c10 = c010 + (c110 - c010) * tx;
    const float c01 = c001 + (c101 - c001) * tx, c11 = c011 + (c111 - c011) * tx;
    const float c0 = c00 + (c10 - c00) * ty, c1 = c01 + (c11 - c01) * ty;
    return c0 + (c1 - c0) * tz;
}

__device__ __forceinline__ float grid_lookup(const float *grid, const Medium &m, V3 uvw)
{
    return grid_trilinear(grid + m.grid_offset, m.res_x, m.res_y, m.res_z, 1, 0, uvw);
}

struct MediumSample
{
    bool scattered;
    V3 position;
    V3 color;      // phase-function colour at the scattering point (the medium's albedo)
    float g;       // Henyey-Greenstein asymmetry
};

// ---------------------------------------------------------------- volume primitives
// VolumePrimitiveMedium (core/btrc/core/volume.cpp:112-197) over the volume BVH
// (core/btrc/core/volume/bvh.cpp:127-262) and the per-overlap delta / ratio tracking of
// volume::Aggregate (core/btrc/core/volume/aggregate.cpp:131-252). The reference selects
// an overlap through a trie of volume-id sequences only to reach code generated per
// overlap set; here the set itself (at most 4 ids) is carried, so no trie is needed.

constexpr uint32_t MAX_VOLUME_SEGMENTS = 1u << 16;

__device__ __forceinline__ V3 vrow(const float *p)
{
    return V3(p[0], p[1], p[2]);
}

// VolumePrimitive::world_pos_to_uvw (core/btrc/core/volume.cpp:45-52)
__device__ __forceinline__ V3 vol_uvw(const VolumePrim &v, V3 p)
{
    const V3 op = p - vrow(v.o);
    return V3(dot(op, vrow(v.x)) * v.x_inv_len2, dot(op, vrow(v.y)) * v.y_inv_len2, dot(op, vrow(v.z)) * v.z_inv_len2);
}

// BVH::is_in_prim (core/btrc/core/volume/bvh.cpp:269-278)
__device__ __forceinline__ bool vol_contains(const VolumePrim &v, V3 p)
{
    const V3 op = p - vrow(v.o);
    const float u = dot(op, vrow(v.xd)), w = dot(op, vrow(v.yd)), x = dot(op, vrow(v.zd));
    return 0.0f <= u && u <= 1.0f && 0.0f <= w && w <= 1.0f && 0.0f <= x && x <= 1.0f;
}

__device__ __forceinline__ bool vol_node_contains(const VolNode &n, V3 p)
{
    return n.lower[0] <= p.x && p.x <= n.upper[0] && n.lower[1] <= p.y && p.y <= n.upper[1] && n.lower[2] <= p.z &&
           p.z <= n.upper[2];
}

// BVH::intersect_ray_aabb (core/btrc/core/volume/bvh.cpp:287-294)
__device__ __forceinline__ bool vol_node_hit(const VolNode &n, V3 o, V3 inv_d, float t_max)
{
    const float nx = inv_d.x * (n.lower[0] - o.x), fx = inv_d.x * (n.upper[0] - o.x);
    const float ny = inv_d.y * (n.lower[1] - o.y), fy = inv_d.y * (n.upper[1] - o.y);
    const float nz = inv_d.z * (n.lower[2] - o.z), fz = inv_d.z * (n.upper[2] - o.z);
    const float t0 = fmaxf(fmaxf(0.0f, fminf(nx, fx)), fmaxf(fminf(ny, fy), fminf(nz, fz)));
    const float t1 = fminf(fminf(t_max, fmaxf(nx, fx)), fminf(fmaxf(ny, fy), fmaxf(nz, fz)));
    return t0 <= t1;
}

// BVH::find_closest_intersection for one box (core/btrc/core/volume/bvh.cpp:296-327):
// the first boundary crossing in (0, t_max) of the segment p + t d, or -1
__device__ __forceinline__ float vol_box_crossing(const VolumePrim &v, V3 p, V3 d, float t_max)
{
    const V3 op = p - vrow(v.o);
    float t0 = 0.0f, t1 = t_max;
    const float *axes[3] = { v.xd, v.yd, v.zd };
#pragma unroll
    for(int a = 0; a < 3; ++a)
    {
        const V3 dd2 = vrow(axes[a]);
        const float opd = dot(op, dd2), dd = dot(d, dd2);
        const float nd = (0.0f - opd) / dd, fd = (1.0f - opd) / dd;
        t0 = fmaxf(t0, fminf(nd, fd));
        t1 = fminf(t1, fmaxf(nd, fd));
    }
    if(t0 > t1)
        return -1.0f;
    if(t0 > 0)
        return t0;
    if(t1 < t_max)
        return t1;
    return -1.0f;
}

// the nearest volume-box boundary strictly inside the segment a -> b
__device__ bool vol_next_boundary(const DevScene &S, V3 a, V3 b, V3 &out)
{
    const V3 dir = b - a;
    const V3 inv(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    float best = MAX_FLOAT, t_max = 1.0f;
    uint32_t stack[VOL_STACK];
    int top = 0;
    stack[top++] = 0;
    while(top > 0)
    {
        const VolNode &n = S.volume_nodes[stack[--top]];
        if(n.prim_beg >= 0)
        {
            for(int i = n.prim_beg; i < n.prim_end; ++i)
            {
                const float t = vol_box_crossing(S.volumes[i], a, dir, t_max);
                if(t >= 0.0f)
                {
                    best = fminf(best, t);
                    t_max = best;
                }
            }
        }
        else
        {
            for(int c = 0; c < 2; ++c)
                if(top < VOL_STACK && vol_node_hit(S.volume_nodes[n.prim_end + c], a, inv, t_max))
                    stack[top++] = static_cast<uint32_t>(n.prim_end + c);
        }
    }
    if(best > 10.0f)
        return false;
    out = a * (1.0f - best) + b * best;
    return true;
}

// volumes containing p (BVH::get_overlap, core/btrc/core/volume/bvh.cpp:197-262): at most
// VOL_MAX_OVERLAP of them, by ascending id; `slot` indexes S.volumes
struct VolOverlap
{
    int count;
    int slot[VOL_MAX_OVERLAP];
};

__device__ VolOverlap vol_overlap(const DevScene &S, V3 p)
{
    VolOverlap r;
    r.count = 0;
    int ids[VOL_MAX_OVERLAP];
    uint32_t stack[VOL_STACK];
    int top = 0;
    stack[top++] = 0;
    while(top > 0)
    {
        const VolNode &n = S.volume_nodes[stack[--top]];
        if(n.prim_beg >= 0)
        {
            for(int i = n.prim_beg; i < n.prim_end; ++i)
            {
                const VolumePrim &v = S.volumes[i];
                if(!vol_contains(v, p))
                    continue;
                const int id = v.id;
                if(r.count == VOL_MAX_OVERLAP && id >= ids[VOL_MAX_OVERLAP - 1])
                    continue;
                int j = r.count < VOL_MAX_OVERLAP ? r.count++ : VOL_MAX_OVERLAP - 1;
                while(j > 0 && ids[j - 1] > id)
                {
                    ids[j] = ids[j - 1];
                    r.slot[j] = r.slot[j - 1];
                    --j;
                }
                ids[j] = id;
                r.slot[j] = i;
            }
        }
        else
        {
            for(int c = 0; c < 2; ++c)
                if(top < VOL_STACK && vol_node_contains(S.volume_nodes[n.prim_end + c], p))
                    stack[top++] = static_cast<uint32_t>(n.prim_end + c);
        }
    }
    return r;
}

__device__ __forceinline__ float vol_sigma(const DevScene &S, const VolumePrim &v, V3 uvw)
{
    if(v.sigma_offset < 0)
        return v.sigma_const;
    return grid_trilinear(S.grids + v.sigma_offset, v.sres[0], v.sres[1], v.sres[2], 1, 0, uvw);
}

// Texture3D::sample_spectrum: a 1-channel array texture reads back as (v, 0, 0), the
// missing channels of a one-component CUDA texture fetch
__device__ __forceinline__ V3 vol_albedo(const DevScene &S, const VolumePrim &v, V3 uvw)
{
    if(v.albedo_offset < 0)
        return vrow(v.albedo_const);
    const float *g = S.grids + v.albedo_offset;
    if(v.albedo_channels == 1)
        return V3(grid_trilinear(g, v.ares[0], v.ares[1], v.ares[2], 1, 0, uvw), 0.0f, 0.0f);
    return V3(grid_trilinear(g, v.ares[0], v.ares[1], v.ares[2], 3, 0, uvw),
              grid_trilinear(g, v.ares[0], v.ares[1], v.ares[2], 3, 1, uvw),
              grid_trilinear(g, v.ares[0], v.ares[1], v.ares[2], 3, 2, uvw));
}

__device__ __forceinline__ float overlap_inv_max(const DevScene &S, const VolOverlap &ov)
{
    float m = 0.0f;
    for(int k = 0; k < ov.count; ++k)
        m += S.volumes[ov.slot[k]].sigma_max;
    return 1.0f / fmaxf(m, 0.01f);
}

// Aggregate::sample_scattering_in_overlap (core/btrc/core/volume/aggregate.cpp:155-219)
__device__ bool vol_sample_overlap(const DevScene &S, const VolOverlap &ov, V3 a, V3 b, DSampler &smp, V3 &pos,
                                   V3 &color)
{
    const float inv_max = overlap_inv_max(S, ov);
    V3 ua[VOL_MAX_OVERLAP], ub[VOL_MAX_OVERLAP];
    for(int k = 0; k < ov.count; ++k)
    {
        ua[k] = vol_uvw(S.volumes[ov.slot[k]], a);
        ub[k] = vol_uvw(S.volumes[ov.slot[k]], b);
    }
    const float t_max = length(b - a);
    float t = 0.0f;
    for(uint32_t it = 0; it < MAX_TRACKING_STEPS; ++it)
    {
        t += -logf(1.0f - smp.get1d()) * inv_max;
        if(t >= t_max)
            return false;
        const float tf = t / t_max;
        float dens[VOL_MAX_OVERLAP];
        V3 uvw[VOL_MAX_OVERLAP];
        float sum = 0.0f;
        for(int k = 0; k < ov.count; ++k)
        {
            uvw[k] = ua[k] * (1.0f - tf) + ub[k] * tf;
            dens[k] = vol_sigma(S, S.volumes[ov.slot[k]], uvw[k]);
            sum += dens[k];
        }
        if(smp.get1d() < sum * inv_max)
        {
            pos = a * (1.0f - tf) + b * tf;
            V3 alb(0.0f);
            for(int k = 0; k < ov.count; ++k)
                alb = alb + (dens[k] / sum) * vol_albedo(S, S.volumes[ov.slot[k]], uvw[k]);
            color = alb;
            return true;
        }
    }
    return false;
}

// Aggregate::tr_in_overlap (core/btrc/core/volume/aggregate.cpp:221-252)
__device__ float vol_tr_overlap(const DevScene &S, const VolOverlap &ov, V3 a, V3 b, DSampler &smp)
{
    const float inv_max = overlap_inv_max(S, ov);
    V3 ua[VOL_MAX_OVERLAP], ub[VOL_MAX_OVERLAP];
    for(int k = 0; k < ov.count; ++k)
    {
        ua[k] = vol_uvw(S.volumes[ov.slot[k]], a);
        ub[k] = vol_uvw(S.volumes[ov.slot[k]], b);
    }
    const float t_max = length(b - a);
    float result = 1.0f, t = 0.0f;
    for(uint32_t it = 0; it < MAX_TRACKING_STEPS; ++it)
    {
        t += -logf(1.0f - smp.get1d()) * inv_max;
        if(t >= t_max)
            break;
        const float tf = t / t_max;
        float sum = 0.0f;
        for(int k = 0; k < ov.count; ++k)
            sum += vol_sigma(S, S.volumes[ov.slot[k]], ua[k] * (1.0f - tf) + ub[k] * tf);
        result *= 1.0f - sum * inv_max;
    }
    return result;
}

// VolumePrimitiveMedium::sample (core/btrc/core/volume.cpp:112-160): walk the segment
// from one box boundary to the next, tracking inside each overlap region; g = 0
__device__ __noinline__ MediumSample volumes_sample(const DevScene &S, V3 a, V3 b, DSampler &smp)
{
    MediumSample r;
    r.scattered = false;
    r.g = 0.0f;
    V3 o = a;
    const V3 d = normalize(b - a);
    for(uint32_t seg = 0; seg < MAX_VOLUME_SEGMENTS; ++seg)
    {
        if(dot(b - o, d) <= 0.0f || length_square(b - o) < 0.00001f)
            break;
        V3 inct;
        if(!vol_next_boundary(S, o, b, inct))
            inct = b;
        const VolOverlap ov = vol_overlap(S, 0.5f * (o + inct));
        if(ov.count != 0 && vol_sample_overlap(S, ov, o, inct, smp, r.position, r.color))
        {
            r.scattered = true;
            break;
        }
        o = inct + 0.001f * d;
    }
    return r;
}

// VolumePrimitiveMedium::tr (core/btrc/core/volume.cpp:162-197)
__device__ __noinline__ float volumes_tr(const DevScene &S, V3 a, V3 b, DSampler &smp)
{
    float result = 1.0f;
    V3 o = a;
    const V3 d = normalize(b - a);
    for(uint32_t seg = 0; seg < MAX_VOLUME_SEGMENTS; ++seg)
    {
        if(dot(b - o, d) <= 0.0f || length_square(b - o) < 0.0001f)
            break;
        V3 inct;
        if(!vol_next_boundary(S, o, b, inct))
            inct = b;
        const VolOverlap ov = vol_overlap(S, 0.5f * (o + inct));
        if(ov.count != 0)
            result *= vol_tr_overlap(S, ov, o, inct, smp);
        o = inct + 0.001f * d;
    }
    return result;
}

// HetergeneousMedium::sample (builtin/btrc/builtin/medium/hetergeneous.cpp:25-73) and the
// homogeneous variant; TransformMedium maps a, b to the medium's local frame first
// (core/btrc/core/medium.cpp:98-129)
__device__ MediumSample medium_sample(const DevScene &S, const Medium &m, V3 a, V3 b, DSampler &smp)
{
    MediumSample r;
    r.scattered = false;
    if(m.type == MED_VACUUM)
        return r;
    if(m.type == MED_VOLUMES)
        return volumes_sample(S, a, b, smp);
    r.color = V3(m.albedo[0], m.albedo[1], m.albedo[2]);
    r.g = m.g;
    const float t_max = length(b - a);
    if(m.type == MED_HOMOGENEOUS)
    {
        const float st = -logf(1.0f - smp.get1d()) / m.sigma_t_const;
        if(st < t_max)
        {
            r.scattered = true;
            r.position = a + normalize(b - a) * st;
        }
        return r;
    }
    const float inv_max = 1.0f / m.sigma_max;
    const V3 la = V3(0.5f) + 0.5f * aff_point(m.w2l, a);
    const V3 lb = V3(0.5f) + 0.5f * aff_point(m.w2l, b);
    const V3 lstep = (lb - la) / t_max;
    const V3 wstep = (b - a) / t_max;
    float t = 0.0f;
    for(uint32_t it = 0; it < MAX_TRACKING_STEPS; ++it)
    {
        t += -logf(1.0f - smp.get1d()) * inv_max;
        if(t >= t_max)
            break;
        const V3 uvw = la + t * lstep;
        const float density = grid_lookup(S.grids, m, uvw);
        if(smp.get1d() < density * inv_max)
        {
            r.scattered = true;
            r.position = a + t * wstep;
            break;
        }
    }
    return r;
}

// ratio-tracking transmittance (hetergeneous.cpp:75-106); homogeneous is analytic
__device__ V3 medium_tr(const DevScene &S, const Medium &m, V3 a, V3 b, DSampler &smp)
{
    if(m.type == MED_VACUUM)
        return V3(1.0f);
    if(m.type == MED_VOLUMES)
        return V3(volumes_tr(S, a, b, smp));
    const float t_max = length(b - a);
    if(m.type == MED_HOMOGENEOUS)
    {
        // the reference attenuates by absorption only (homogeneous.cpp:49-62)
        const V3 sigma_a = m.sigma_t_const * (V3(1.0f) - V3(m.albedo[0], m.albedo[1], m.albedo[2]));
        const V3 e = -t_max * sigma_a;
        return V3(expf(e.x), expf(e.y), expf(e.z));
    }
    const float inv_max = 1.0f / m.sigma_max;
    const V3 la = V3(0.5f) + 0.5f * aff_point(m.w2l, a);
    const V3 lb = V3(0.5f) + 0.5f * aff_point(m.w2l, b);
    const V3 lstep = (lb - la) / t_max;
    float result = 1.0f, t = 0.0f;
    for(uint32_t it = 0; it < MAX_TRACKING_STEPS; ++it)
    {
        t += -logf(1.0f - smp.get1d()) * inv_max;
        if(t >= t_max)
            break;
        const V3 uvw = la + t * lstep;
        result *= 1.0f - grid_lookup(S.grids, m, uvw) * inv_max;
    }
    return V3(result);
}

__device__ __forceinline__ float henyey_greenstein(float g, float u)
{
    const float g2 = g * g;
    const float dem = 1.0f + g2 - 2.0f * (g * u);
    return (1.0f - g2) / (4.0f * PI * dem * sqrtf(dem));
}

// ---------------------------------------------------------------- kernels

// Starts a bounce of the given parity. Writes its fields one by one: the shadow kernel of
// the previous bounce (other parity) may still be running and updating its own cursor.
__global__ void k_control(Counters *c, uint32_t capacity, uint64_t total, int parity)
{
    const uint32_t survivors = c->next_active;
    const uint64_t generated = c->generated;
    const uint64_t remaining = total - generated;
    const uint64_t room = capacity - survivors;
    const uint32_t n_new = static_cast<uint32_t>(remaining < room ? remaining : room);
    const uint32_t active = survivors + n_new;
    c->shadow_rays += c->shadow_n[parity];
    c->shadow_n[parity] = 0;
    c->shadow_cursor[parity] = 0;
    c->slot_base = survivors;
    c->n_new = n_new;
    c->gen_base = generated;
    c->generated = generated + n_new;
    c->active = active;
    c->ext_rays += active;
    c->next_active = 0;
    c->trace_cursor = 0;
    c->hit_count = 0;
    c->miss_count = 0;
    if(active > 0)
        ++c->iterations;
}

// which scenes of a merged batch still have paths in the queue: live[s] = 1 (warp lanes of
// one scene store once)
__global__ void k_batch_live(DevRender R, const F4 *__restrict__ rad_pixel, const Counters *__restrict__ c,
                             uint8_t *__restrict__ live)
{
    const uint32_t n = c->next_active;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t end = (n + 31u) & ~31u;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < end; i += stride)
    {
        const int s = i < n ? R.row_scene[__float_as_uint(rad_pixel[i].w) >> 16] : -1;
        const uint32_t same = __match_any_sync(0xffffffffu, s);
        if(s >= 0 && static_cast<uint32_t>(s) < R.batch_count && (threadIdx.x & 31u) == __ffs(same) - 1u)
            live[s] = 1;
    }
}

// the scene of global camera path g in a merged batch: the last with path_begin <= g
__device__ __forceinline__ int batch_scene_of_path(const DevRender &R, uint64_t g)
{
    int lo = 0, hi = static_cast<int>(R.batch_count) - 1;
    while(lo < hi)
    {
        const int mid = (lo + hi + 1) >> 1;
        if(R.batch[mid].path_begin <= g)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

template<bool MULTI>
__global__ void __launch_bounds__(BLOCK) k_generate(DevRender R_in, PathSoA P, float4 *film, const Counters *cnt,
                                                    int vacuum_in)
{
    const uint32_t n = cnt->n_new;
    const uint32_t slot_base = cnt->slot_base;
    const uint64_t gen_base = cnt->gen_base;
    const uint32_t stride = gridDim.x * blockDim.x;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        // a merged batch: the path's scene supplies camera, film and sampler; its film is
        // a band of rows of the combined film
        uint64_t g = gen_base + i;
        uint32_t row_base = 0;
        int vacuum_medium = vacuum_in;
        DevRender Rb;
        if(MULTI)
        {
            const BatchScene &b = R_in.batch[batch_scene_of_path(R_in, g)];
            Rb = b.R;
            g -= b.path_begin;
            row_base = b.row_base;
            vacuum_medium = b.vacuum_medium;
        }
        const DevRender &R = MULTI ? Rb : R_in;
        const uint64_t pixel_count = static_cast<uint64_t>(R.width) * R.height;
        uint64_t pixel, sample;
        if(!R.tile)
        {
            pixel = g % pixel_count;
            sample = g / pixel_count;
        }
        else
        {
            pixel = g / R.spp;
            sample = g % R.spp;
        }
        const uint32_t px = static_cast<uint32_t>(pixel % R.width);
        const uint32_t py = static_cast<uint32_t>(pixel / R.width);
        DSampler smp;
        smp.type = R.sampler;
        smp.s = sampler_init(R.sampler, R.halton, px, py, static_cast<uint32_t>(sample) + R.sample_offset);
        float fx, fy;
        if(R.filter == FILTER_GAUSSIAN)
        {
            // GaussianFilter::sample (builtin/btrc/builtin/film_filter/gaussian.cpp:54-66)
            const uint32_t cell = alias_sample(R.filter_table, FILTER_GRID * FILTER_GRID, smp.get1d());
            const uint32_t gy = cell / FILTER_GRID, gx = cell % FILTER_GRID;
            const float r = R.filter_radius, w = 2 * r / FILTER_GRID;
            const float x0 = -r + w * static_cast<float>(gx), x1 = -r + w * static_cast<float>(gx + 1);
            const float y0 = -r + w * static_cast<float>(gy), y1 = -r + w * static_cast<float>(gy + 1);
            fx = lerpf(x0, x1, smp.get1d());
            fy = lerpf(y0, y1, smp.get1d());
        }
        else
        {
            fx = smp.get1d() - 0.5f;
            fy = smp.get1d() - 0.5f;
        }
        const float film_x = (static_cast<float>(px) + 0.5f + fx) / static_cast<float>(R.width);
        const float film_y = (static_cast<float>(py) + 0.5f + fy) / static_cast<float>(R.height);
        (void)smp.get1d();  // time sample
        // PinholeCamera::generate_ray_inline (builtin/btrc/builtin/camera/pinhole.cpp:84-99)
        const V3 dst = R.cam_lbc + film_x * R.cam_fx + film_y * R.cam_fy;
        const V3 dir = normalize(dst - R.cam_eye);
        const uint32_t row = py + row_base;
        const uint32_t pix = px | (row << 16);
        atomicAdd(&film[static_cast<size_t>(row) * R_in.width + px].w, 1.0f);
        const uint32_t s = slot_base + i;
        P.beta_depth[s] = F4{ 1.0f, 1.0f, 1.0f, __int_as_float(0) };
        P.rad_pixel[s] = F4{ 0.0f, 0.0f, 0.0f, __uint_as_float(pix) };
        P.sampler[s] = smp.s;
        P.ray_o[s] = F4{ R.cam_eye.x, R.cam_eye.y, R.cam_eye.z, __int_as_float(vacuum_medium) };
        P.ray_d[s] = F4{ dir.x, dir.y, dir.z, MAX_FLOAT };
        P.bsdf_le[s] = F4{ 1.0f, 1.0f, 1.0f, -1.0f };
    }
}

// TWO: the scene's two-level form (no counting, no merged batch)
template<bool COUNT, bool MULTI = false, bool TWO = false>
__global__ void __launch_bounds__(TRAVERSE_BLOCK) k_trace(DevScene S, PathSoA P, uint32_t *flags, HitDetail *hits,
                                               Counters *cnt, DevRender R)
{
    const uint32_t n = cnt->active;
    uint64_t nv = 0, tv = 0;
    auto fetch = [&](uint32_t i, float *o, float *d, float &t1, uint32_t &root) {
        const F4 ro = P.ray_o[i], rd = P.ray_d[i];
        o[0] = ro.x; o[1] = ro.y; o[2] = ro.z;
        d[0] = rd.x; d[1] = rd.y; d[2] = rd.z;
        t1 = rd.w;
        if(MULTI)
            root = R.batch[R.row_scene[__float_as_uint(P.rad_pixel[i].w) >> 16]].root;
    };
    auto emit = [&](uint32_t i, const ClosestResult &c) {
        flags[i] = c.hit ? (c.inst | HIT_BIT) : 0u;
        hits[i] = HitDetail{ c.t, c.prim, c.b1, c.b2 };
    };
    if constexpr(TWO)
        traverse_refill<false, false, true>(reinterpret_cast<const float4 *>(S.nodes),
                                            reinterpret_cast<const float4 *>(S.tris), S.node_count, &cnt->trace_cursor,
                                            n, REFILL_LANES, &cnt->err, fetch, emit, nullptr, nullptr, S.tri_round,
                                            two_level_view(S));
    else
        traverse_refill<false, COUNT>(reinterpret_cast<const float4 *>(S.nodes),
                                      reinterpret_cast<const float4 *>(S.tris), S.node_count, &cnt->trace_cursor, n,
                                      REFILL_LANES, &cnt->err, fetch, emit, &nv, &tv, S.tri_round);
    if(COUNT && !TWO)
    {
        for(int off = 16; off > 0; off >>= 1)
        {
            nv += __shfl_down_sync(0xffffffffu, nv, off);
            tv += __shfl_down_sync(0xffffffffu, tv, off);
        }
        if(lane_id() == 0)
        {
            atomicAdd(reinterpret_cast<unsigned long long *>(&cnt->node_visits), static_cast<unsigned long long>(nv));
            atomicAdd(reinterpret_cast<unsigned long long *>(&cnt->tri_tests), static_cast<unsigned long long>(tv));
        }
    }
}

// Shade order: a permutation of the queue slots with the paths that hit a surface first
// (in slot order) and the misses after them, so that the shade kernel's warps run the
// surface code with full lanes and the short miss code apart from it. Each block takes
// ORDER_ITEMS consecutive slots per thread, scans the counts in shared memory and claims
// its ranges with one atomic per kind. The shade kernel checks every path's flags itself,
// so the order only groups work; it never changes a result.
constexpr uint32_t ORDER_ITEMS = 8;

__global__ void __launch_bounds__(BLOCK) k_order(const uint32_t *__restrict__ flags, uint32_t *__restrict__ order,
                                                 Counters *cnt)
{
    __shared__ uint32_t s_warp[BLOCK / 32];
    __shared__ uint32_t s_base[2];
    const uint32_t n = cnt->active;
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const uint32_t chunk = BLOCK * ORDER_ITEMS;
    for(uint32_t c0 = blockIdx.x * chunk; c0 < n; c0 += gridDim.x * chunk)
    {
        const uint32_t first = c0 + threadIdx.x * ORDER_ITEMS;
        uint32_t hitbits = 0, valid = 0;
#pragma unroll
        for(uint32_t k = 0; k < ORDER_ITEMS; ++k)
            if(first + k < n)
            {
                ++valid;
                if(flags[first + k] & HIT_BIT)
                    hitbits |= 1u << k;
            }
        // hits in the low half, misses in the high half (at most BLOCK * ORDER_ITEMS each)
        const uint32_t v = static_cast<uint32_t>(__popc(hitbits)) | ((valid - __popc(hitbits)) << 16);
        uint32_t x = v;
#pragma unroll
        for(int off = 1; off < 32; off <<= 1)
        {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
            if(lane >= static_cast<uint32_t>(off))
                x += y;
        }
        if(lane == 31)
            s_warp[warp] = x;
        __syncthreads();
        if(warp == 0)
        {
            const uint32_t w = lane < BLOCK / 32 ? s_warp[lane] : 0u;
            uint32_t t = w;
#pragma unroll
            for(int off = 1; off < 32; off <<= 1)
            {
                const uint32_t y = __shfl_up_sync(0xffffffffu, t, off);
                if(lane >= static_cast<uint32_t>(off))
                    t += y;
            }
            if(lane < BLOCK / 32)
                s_warp[lane] = t - w;
            if(lane == 31)
            {
                s_base[0] = (t & 0xffffu) ? atomicAdd(&cnt->hit_count, t & 0xffffu) : 0u;
                s_base[1] = (t >> 16) ? atomicAdd(&cnt->miss_count, t >> 16) : 0u;
            }
        }
        __syncthreads();
        const uint32_t excl = s_warp[warp] + x - v;
        uint32_t hpos = s_base[0] + (excl & 0xffffu);
        uint32_t mpos = s_base[1] + (excl >> 16);
#pragma unroll
        for(uint32_t k = 0; k < ORDER_ITEMS; ++k)
            if(first + k < n)
            {
                if(hitbits & (1u << k))
                    order[hpos++] = first + k;
                else
                    order[n - 1u - mpos++] = first + k;
            }
        __syncthreads();
    }
}

// MediumPipeline (builtin/btrc/builtin/renderer/wavefront/medium.cpp:28-249). Four blocks
// per SM (64 registers, a few hundred bytes of spills): the tracking loop waits on
// dependent density fetches, and the volume frame (256^3 grid, 1024^2, 64 spp) ran in
// 832 ms against 856 ms at three blocks (80 registers) and 841-858 ms at five
__global__ void __launch_bounds__(BLOCK, 4) k_medium(DevScene S, DevRender R, PathSoA P, PathSoA N, ShadowSoA SH, int shq,
                                                  uint32_t *flags, const HitDetail *hits, float4 *film, Counters *cnt)
{
    const uint32_t n = cnt->active;
    const uint32_t stride = gridDim.x * blockDim.x;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        const uint32_t flag = flags[i];
        const F4 ro = P.ray_o[i], rd = P.ray_d[i];
        const V3 o = v3(ro), d = v3(rd);
        const int ray_medium = __float_as_int(ro.w);
        int medium_id;
        V3 end;
        if(flag & HIT_BIT)
        {
            const HitDetail h = hits[i];
            const Instance &inst = S.instances[flag & INST_MASK];
            const Geometry g = S.geometries[inst.geometry];
            const V3 ln = v3(ldf4(S.shade + static_cast<size_t>(g.tri_offset + h.prim) * SHADE_F4 + 2));
            const V3 nor = aff_normal(inst.w2l, ln);
            const int inner = static_cast<int>(inst.media & 0xffffu), outer = static_cast<int>(inst.media >> 16);
            const int inct_medium = dot(d, nor) < 0 ? outer : inner;
            medium_id = min(inct_medium, ray_medium);
            end = offset_dir(o + h.t * d, nor, -d);
        }
        else
        {
            medium_id = S.vacuum_medium;
            end = o + normalize(d) * S.world_diagonal;
        }
        P.ray_o[i].w = __int_as_float(medium_id);
        const Medium &m = S.media[medium_id];
        if(m.type == MED_VACUUM)
            continue;

        DSampler smp;
        smp.type = R.sampler;
        smp.s = P.sampler[i];
        const MediumSample ms = medium_sample(S, m, o, end, smp);
        const V3 tr = medium_tr(S, m, o, end, smp);
        F4 ble = P.bsdf_le[i];
        ble.x *= tr.x;
        ble.y *= tr.y;
        ble.z *= tr.z;
        P.bsdf_le[i] = ble;
        if(!ms.scattered)
        {
            P.sampler[i] = smp.s;
            continue;
        }
        flags[i] = flag | SCATTER_BIT;
        const F4 bd = P.beta_depth[i], rp = P.rad_pixel[i];
        V3 beta = v3(bd);
        const int depth = __float_as_int(bd.w);
        const uint32_t pixel = __float_as_uint(rp.w);
        const V3 path_rad = v3(rp);
        if(russian_roulette(beta, depth, smp, R))
        {
            splat(film, pixel, R.width, path_rad);
            continue;
        }
        const V3 albedo = ms.color;
        LightSample ls = sample_light(S, ms.position, V3(0, 0, 1), false, smp);
        if(ls.success)
        {
            // HG eval/pdf with u = -cos(wi, wo)
            const V3 wo = -d;
            const float u = -dot(normalize(ls.d), normalize(wo));
            const float ph = henyey_greenstein(ms.g, u);
            ls.li = ls.li * beta * (albedo * ph) / (ph + ls.light_pdf);
        }
        // HenyeyGreensteinPhaseShader::sample (core/btrc/core/medium.cpp:32-64)
        float s0, s1, s2;
        smp.get3d(s0, s1, s2);
        const float g = ms.g;
        const float s = s0 + s0 - 1;
        float u;
        if(fabsf(g) < 0.001f)
            u = s;
        else
        {
            const float g2 = g * g;
            u = (1.0f + g2 - sqrf((1.0f - g2) / (1.0f + g * s))) / (g + g);
        }
        const float cos_theta = -u;
        const float sin_theta = cos2sin(cos_theta);
        float sp, cp;
        sincos_pi(2.0f * s1, sp, cp);
        const V3 lwi(sin_theta * sp, sin_theta * cp, cos_theta);
        const float phase_val = henyey_greenstein(g, u);
        const V3 phase = albedo * phase_val;
        V3 ndir = Frame::from_z(-d).local_to_global(lwi);
        (void)s2;
        if(ls.success)
        {
            const uint32_t k = queue_append(&cnt->shadow_n[shq]);
            const int smed = ls.t1 > 1 ? S.vacuum_medium : medium_id;
            SH.o[k] = f4(ls.o, __uint_as_float(pixel));
            SH.d[k] = f4(ls.d, ls.t1);
            SH.beta[k] = f4(ls.li, __int_as_float(smed));
            SamplerState ss;
            pcg32_seed(ss.a, ss.b, shadow_stream_seed(P.sampler[i], SHADOW_FROM_MEDIUM), PCG_STREAM);
            SH.sampler[k] = ss;
        }
        if(!is_zero(phase))
        {
            ndir = normalize(ndir);
            const V3 beta_le = beta * phase;
            beta = beta_le / phase_val;
            const uint32_t k = queue_append(&cnt->next_active);
            N.beta_depth[k] = f4(beta, __int_as_float(depth + 1));
            N.rad_pixel[k] = f4(path_rad, __uint_as_float(pixel));
            N.sampler[k] = smp.s;
            N.ray_o[k] = f4(ms.position, __int_as_float(medium_id));
            N.ray_d[k] = f4(ndir, MAX_FLOAT);
            N.bsdf_le[k] = f4(beta_le, phase_val);
        }
        else
            splat(film, pixel, R.width, path_rad);
    }
}

// Texture2D parameters of a material sampled at the hit's texture coordinate (every
// material creator's context.create<Texture2D>), and the normal map's local normal
// 2 tex - 1 (builtin/btrc/builtin/material/utils/normal_map.cpp:13-21). Returned by value
// so that the untextured path keeps the material and frame in registers.
struct MaterialTexValues
{
    float p[16];
    uint32_t mask;    // bit k: p[k] comes from a texture
    int has_normal;
    V3 normal;        // normal-map direction in the shading frame
};

__device__ __forceinline__ MaterialTexValues eval_material_textures(const DevScene &S, int row, float tu, float tv)
{
    MaterialTexValues r;
    r.mask = 0;
    r.has_normal = 0;
    const MaterialTex &mt = S.material_tex[row];
    const TexTables T = tex_tables(S);
    if(mt.prog[0] >= 0)
    {
        const V3 c = tex_eval(T, mt.prog[0], tu, tv);
        r.p[0] = c.x;
        r.p[1] = c.y;
        r.p[2] = c.z;
        r.mask |= 7u;
    }
    for(int k = 3; k < 16; ++k)
        if(mt.prog[k] >= 0)
        {
            r.p[k] = tex_eval(T, mt.prog[k], tu, tv).x;
            r.mask |= 1u << k;
        }
    if(mt.normal >= 0)
    {
        r.has_normal = 1;
        r.normal = 2.0f * tex_eval(T, mt.normal, tu, tv) - V3(1.0f);
    }
    return r;
}

// ShadePipeline (builtin/btrc/builtin/renderer/wavefront/shade.cpp:29-235)
// Radiance-cache query of a surface vertex: position, direction towards the previous
// vertex, shading normal (normal-mapped), roughness and diffuse albedo. Delta surfaces
// (mirror, glass, invisible) get no query: the path continues through them.
template<bool TEX>
__device__ __forceinline__ bool nrc_query_at(const DevScene &S, const SurfacePoint &sp, const Instance &inst, V3 wo,
                                             float *q)
{
    Material mat = S.materials[inst.material];
    if(mat.type == MAT_MIRROR || mat.type == MAT_GLASS || mat.type == MAT_INVISIBLE)
        return false;
    Frame shading = sp.frame.rotate_to_new_z(sp.interp_z);
    if(TEX && mat.tex >= 0)
    {
        const MaterialTexValues tv = eval_material_textures(S, mat.tex, sp.tu, sp.tv);
#pragma unroll
        for(int k = 0; k < 16; ++k)
            if(tv.mask & (1u << k))
                mat.p[k] = tv.p[k];
        if(tv.has_normal)
            shading = shading.rotate_to_new_z(normalize(shading.local_to_global(tv.normal)));
    }
    const V3 n = shading.z;
    float rough = 1.0f;
    V3 alb(mat.p[0], mat.p[1], mat.p[2]);
    if(mat.type == MAT_METAL)
        rough = mat.p[3];
    else if(mat.type == MAT_DISNEY)
        rough = mat.p[4];
    else if(mat.type == MAT_BLACK)
        alb = V3(0.0f);
    q[0] = sp.position.x; q[1] = sp.position.y; q[2] = sp.position.z;
    q[3] = wo.x; q[4] = wo.y; q[5] = wo.z;
    q[6] = n.x; q[7] = n.y; q[8] = n.z;
    q[9] = rough;
    q[10] = alb.x; q[11] = alb.y; q[12] = alb.z;
    return true;
}

// TEX = false compiles the texture evaluation out, so scenes without textured materials
// keep the shade kernel's registers. Two blocks per SM (at most 128 registers a thread):
// the kernel waits on scattered loads, and the occupancy pays for the few spills.
template<bool TEX, bool NRC = false, bool MULTI = false>
__global__ void __launch_bounds__(BLOCK, 2) k_shade(DevScene S_in, DevRender R_in, PathSoA P, PathSoA N, ShadowSoA SH,
                                                    int shq, const uint32_t *flags, const HitDetail *hits,
                                                 const uint32_t *order, float4 *film, Counters *cnt)
{
    const uint32_t n = cnt->active;
    const uint32_t stride = gridDim.x * blockDim.x;
    for(uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride)
    {
        const uint32_t i = order[j];
        const uint32_t flag = flags[i];
        const F4 bd = P.beta_depth[i], rp = P.rad_pixel[i];
        const F4 ro = P.ray_o[i], rd = P.ray_d[i], ble = P.bsdf_le[i];
        const uint32_t pixel = __float_as_uint(rp.w);
        // a merged batch: the path's scene supplies its lights, environment and path-length
        // rules; film splats stay in combined-film coordinates
        DevScene Sb;
        DevRender Rb;
        if(MULTI)
        {
            const BatchScene &b = R_in.batch[R_in.row_scene[pixel >> 16]];
            Sb = S_in;
            Sb.area_lights = S_in.area_lights + b.light_begin;
            Sb.num_area_lights = b.num_area_lights;
            Sb.num_lights = b.num_lights;
            Sb.env = b.env;
            Sb.world_diagonal = b.world_diagonal;
            Sb.vacuum_medium = b.vacuum_medium;
            Rb = R_in;
            Rb.min_depth = b.R.min_depth;
            Rb.max_depth = b.R.max_depth;
            Rb.rr_threshold = b.R.rr_threshold;
            Rb.rr_cont_prob = b.R.rr_cont_prob;
            Rb.sampler = b.R.sampler;
        }
        const DevScene &S = MULTI ? Sb : S_in;
        const DevRender &R = MULTI ? Rb : R_in;
        const V3 o = v3(ro), d = v3(rd), beta_le = v3(ble);
        const float bsdf_pdf = ble.w;
        V3 path_rad = v3(rp);
        const bool scattered = (flag & SCATTER_BIT) != 0;

        if(!(flag & HIT_BIT))
        {
            V3 rad = miss_le(S, d, beta_le, bsdf_pdf);
            if(!scattered)
                rad = rad + path_rad;
            splat(film, pixel, R.width, rad);
            continue;
        }

        const HitDetail h = hits[i];
        const Instance &inst = S.instances[flag & INST_MASK];
        const Geometry geo = S.geometries[inst.geometry];
        const SurfacePoint sp = get_hitinfo(S, o, d, inst, geo.tri_offset + h.prim, h.t, h.b1, h.b2);
        const V3 le = hit_light_le(S, o, d, sp, beta_le, bsdf_pdf, inst.light);
        if(scattered)
        {
            splat(film, pixel, R.width, le);
            continue;
        }
        path_rad = path_rad + le;

        V3 beta = v3(bd);
        const int depth = __float_as_int(bd.w);
        // path spread (Mueller, Rousselle, Novak, Keller, "Real-time Neural Radiance Caching
        // for Path Tracing", 2021, section 4): a(x1..xn) = (sum_{i>=2} sqrt(|x_{i-1} - x_i|^2 /
        // (p(w_i) |cos theta_i|)))^2 against a0 = |x0 - x1|^2 / (4 pi cos theta_1); kept
        // normalised by sqrt(a0), so the path ends once the sum passes sqrt(c)
        float2 spread = make_float2(0.0f, 0.0f);
        bool spread_end = false;
        if(NRC && R.nrc_spread_c > 0.0f)
        {
            const float cosv = fmaxf(fabsf(dot(sp.frame.z, d)), 1e-6f);
            if(depth == 0)
                spread = make_float2(0.0f, h.t / sqrtf(4.0f * PI * cosv));
            else
            {
                spread = R.nrc_spread[shq][i];
                if(bsdf_pdf > 0.0f && spread.y > 0.0f)
                    spread.x += sqrtf(h.t * h.t / (bsdf_pdf * cosv)) / spread.y;
                spread_end = spread.x * spread.x > R.nrc_spread_c;
            }
        }
        if(NRC && (R.nrc_spread_c > 0.0f ? spread_end : depth >= R.nrc_terminate))
        {
            // terminate into the radiance cache at a non-delta vertex: the cache's
            // prediction replaces light sampling and everything after this vertex
            float q[NRC_QUERY_FLOATS];
            if(nrc_query_at<TEX>(S, sp, inst, -d, q))
            {
                const uint32_t k = atomicAdd(R.nrc_count, 1u);
                if(k < R.nrc_cap)
                {
                    for(int j = 0; j < NRC_QUERY_FLOATS; ++j)
                        R.nrc_query[static_cast<size_t>(k) * NRC_QUERY_FLOATS + j] = q[j];
                    R.nrc_weight[k] = make_float4(beta.x, beta.y, beta.z, __uint_as_float(pixel));
                }
                splat(film, pixel, R.width, path_rad);
                continue;
            }
        }
        DSampler smp;
        smp.type = R.sampler;
        smp.s = P.sampler[i];
        if(russian_roulette(beta, depth, smp, R))
        {
            splat(film, pixel, R.width, path_rad);
            continue;
        }

        LightSample ls = sample_light(S, sp.position, sp.frame.z, true, smp);

        Material mat = S.materials[inst.material];
        SurfaceShader sh;
        sh.frame.geometry = sp.frame;
        sh.frame.shading = sp.frame.rotate_to_new_z(sp.interp_z);
        if(TEX && mat.tex >= 0)
        {
            const MaterialTexValues tv = eval_material_textures(S, mat.tex, sp.tu, sp.tv);
#pragma unroll
            for(int k = 0; k < 16; ++k)
                if(tv.mask & (1u << k))
                    mat.p[k] = tv.p[k];
            if(tv.has_normal)
                sh.frame.shading =
                    sh.frame.shading.rotate_to_new_z(normalize(sh.frame.shading.local_to_global(tv.normal)));
        }
        sh.mat = make_material_eval(mat);
        sh.shadow_terminator = mat.shadow_terminator != 0;

        // g-buffer at the first hit (shade.cpp:133-139, 195-202): Shader::albedo and
        // Shader::normal; black / invisible report the geometric normal
        if(depth == 0 && (R.aov_albedo != nullptr || R.aov_normal != nullptr))
        {
            const bool geo_normal = mat.type == MAT_BLACK || mat.type == MAT_INVISIBLE;
            const V3 alb = mat.type == MAT_BLACK ? V3(0.0f)
                           : mat.type == MAT_INVISIBLE ? V3(1.0f)
                                                       : V3(mat.p[0], mat.p[1], mat.p[2]);
            const V3 nrm = geo_normal ? sp.frame.z : sh.frame.shading.z;
            if(R.aov_albedo != nullptr)
                splat(R.aov_albedo, pixel, R.width, alb);
            if(R.aov_normal != nullptr)
                splat(R.aov_normal, pixel, R.width, nrm);
        }

        float u0, u1, u2;
        smp.get3d(u0, u1, u2);
        const V3 wo = -d;
        V3 shadow_f;
        float shadow_pdf;
        CompSample bs = sh.sample_eval(wo, u0, u1, u2, ls.success, ls.d, shadow_f, shadow_pdf);
        if(ls.success)
            ls.success = !is_zero(shadow_f);

        if(ls.success)
        {
            const bool shadow_out = dot(sp.frame.z, ls.d) > 0;
            const bool last_out = dot(sp.frame.z, d) < 0;
            const int inner = static_cast<int>(inst.media & 0xffffu), outer = static_cast<int>(inst.media >> 16);
            const int smed = shadow_out == last_out ? __float_as_int(ro.w) : (shadow_out ? outer : inner);
            const float c = fabsf(dot(normalize(ls.d), sp.frame.z));
            const V3 beta_li = ls.li * beta * shadow_f * c / (shadow_pdf + ls.light_pdf);
            const uint32_t k = queue_append(&cnt->shadow_n[shq]);
            SH.o[k] = f4(ls.o, __uint_as_float(pixel));
            SH.d[k] = f4(ls.d, ls.t1);
            SH.beta[k] = f4(beta_li, __int_as_float(smed));
            if(S.has_media)
            {
                SamplerState ss;
                pcg32_seed(ss.a, ss.b, shadow_stream_seed(P.sampler[i], SHADOW_FROM_SURFACE), PCG_STREAM);
                SH.sampler[k] = ss;
            }
        }

        if(!is_zero(bs.f))
        {
            const V3 ndir = normalize(bs.dir);
            const float c = fabsf(dot(ndir, sp.frame.z));
            const V3 new_beta_le = beta * c * bs.f;
            beta = new_beta_le / bs.pdf;
            const V3 no = offset_dir(sp.position, sp.frame.z, ndir);
            const bool nout = dot(sp.frame.z, ndir) > 0;
            const int nmed = nout ? static_cast<int>(inst.media >> 16) : static_cast<int>(inst.media & 0xffffu);
            const float stored_pdf = bs.is_delta ? -bs.pdf : bs.pdf;
            const uint32_t k = queue_append(&cnt->next_active);
            N.beta_depth[k] = f4(beta, __int_as_float(depth + 1));
            N.rad_pixel[k] = f4(path_rad, __uint_as_float(pixel));
            N.sampler[k] = smp.s;
            N.ray_o[k] = f4(no, __int_as_float(nmed));
            N.ray_d[k] = f4(ndir, MAX_FLOAT);
            N.bsdf_le[k] = f4(new_beta_le, stored_pdf);
            if(NRC && R.nrc_spread_c > 0.0f)
                R.nrc_spread[1 - shq][k] = spread;
        }
        else
            splat(film, pixel, R.width, path_rad);
    }
}

using ShadeKernel = void (*)(DevScene, DevRender, PathSoA, PathSoA, ShadowSoA, int, const uint32_t *,
                             const HitDetail *, const uint32_t *, float4 *, Counters *);

// the shade kernel variant for a scene and render: textured materials, cache termination,
// a merged batch (untextured, no cache)
ShadeKernel shade_kernel(const DevScene &S, const DevRender &R)
{
    if(R.batch)
        return k_shade<false, false, true>;
    const bool tex = S.material_tex != nullptr, nrc = R.nrc_terminate >= 0;
    if(tex)
        return nrc ? k_shade<true, true> : k_shade<true, false>;
    return nrc ? k_shade<false, true> : k_shade<false, false>;
}

// ShadowPipeline (builtin/btrc/builtin/renderer/wavefront/shadow.cpp:24-76): occlusion by
// the warp-refill traversal; unoccluded records splat (times the medium transmittance)
// MEDIA = false compiles the transmittance code out, so the traversal of scenes without
// media keeps its registers
template<bool MEDIA, bool MULTI = false, bool TWO = false>
__global__ void __launch_bounds__(TRAVERSE_BLOCK) k_shadow(DevScene S, DevRender R, ShadowSoA SH, float4 *film,
                                                           Counters *cnt, int shq)
{
    const uint32_t n = cnt->shadow_n[shq];
    auto fetch = [&](uint32_t i, float *o, float *d, float &t1, uint32_t &root) {
        const F4 so = SH.o[i], sd = SH.d[i];
        o[0] = so.x; o[1] = so.y; o[2] = so.z;
        d[0] = sd.x; d[1] = sd.y; d[2] = sd.z;
        t1 = sd.w;
        if(MULTI)
            root = R.batch[R.row_scene[__float_as_uint(so.w) >> 16]].root;
    };
    auto emit = [&](uint32_t i, const ClosestResult &c) {
        if(c.hit)
            return;
        const F4 o = SH.o[i], d = SH.d[i], b = SH.beta[i];
        V3 beta = v3(b);
        if(MEDIA)
        {
            DSampler smp;
            smp.type = SAMPLER_INDEPENDENT;
            smp.s = SH.sampler[i];
            const V3 ro = v3(o), rdv = v3(d);
            if(d.w > 1)
            {
                const Medium &m = S.media[S.vacuum_medium];
                beta = beta * medium_tr(S, m, ro, ro + normalize(rdv) * S.world_diagonal, smp);
            }
            else
            {
                const Medium &m = S.media[__float_as_int(b.w)];
                beta = beta * medium_tr(S, m, ro, ro + rdv * d.w, smp);
            }
        }
        splat(film, __float_as_uint(o.w), R.width, beta);
    };
    if constexpr(TWO)
        traverse_refill<true, false, true>(reinterpret_cast<const float4 *>(S.nodes),
                                           reinterpret_cast<const float4 *>(S.tris), S.node_count,
                                           &cnt->shadow_cursor[shq], n, REFILL_LANES, &cnt->err, fetch, emit, nullptr,
                                           nullptr, S.shadow_round, two_level_view(S));
    else
        traverse_refill<true>(reinterpret_cast<const float4 *>(S.nodes), reinterpret_cast<const float4 *>(S.tris),
                              S.node_count, &cnt->shadow_cursor[shq], n, REFILL_LANES, &cnt->err, fetch, emit, nullptr,
                              nullptr, S.shadow_round);
}

__global__ void k_resolve(const float4 *film, float *rgb, uint32_t pixels)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= pixels)
        return;
    const float4 f = film[i];
    const float inv = f.w > 0 ? 1.0f / f.w : 0.0f;
    rgb[i * 3 + 0] = f.x * inv;
    rgb[i * 3 + 1] = f.y * inv;
    rgb[i * 3 + 2] = f.z * inv;
}

uint64_t *launches_by_stage_ptr(uint64_t *p) { return p; }

int persistent_grid(int block, const void *kernel, int pct = 100)
{
    int dev = 0, sms = 152, per_sm = 4;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
    const int full = sms * (per_sm > 0 ? per_sm : 1);
    const int scaled = pct > 0 && pct < 100 ? full * pct / 100 : full;
    return scaled > 0 ? scaled : 1;
}

// Per-stage event timing for profile mode 1: a pair of events around every launch.
struct StageTimer
{
    std::vector<cudaEvent_t> pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
    size_t used = 0;
    cudaEvent_t get()
    {
        if(used == pool.size())
        {
            cudaEvent_t e;
            cudaEventCreate(&e);
            pool.push_back(e);
        }
        return pool[used++];
    }
    ~StageTimer()
    {
        for(auto e : pool)
            cudaEventDestroy(e);
    }
};

template<typename Launch>
void timed(StageTimer *T, int stage, cudaStream_t st, uint64_t *launches, Launch &&fn)
{
    ++launches[stage];
    if(!T)
    {
        fn();
        return;
    }
    cudaEvent_t a = T->get(), b = T->get();
    cudaEventRecord(a, st);
    fn();
    cudaEventRecord(b, st);
    T->marks.push_back({ stage, { a, b } });
}

void launch_shadow(const DevScene &S, const DevRender &R, RenderBuffers &B, int parity, cudaStream_t st, int grid)
{
    if(R.batch)
        k_shadow<false, true><<<grid, TRAVERSE_BLOCK, 0, st>>>(S, R, B.shadow[parity], B.film, B.counters, parity);
    else if(S.two_level)
    {
        if(S.has_media)
            k_shadow<true, false, true><<<grid, TRAVERSE_BLOCK, 0, st>>>(S, R, B.shadow[parity], B.film, B.counters,
                                                                        parity);
        else
            k_shadow<false, false, true><<<grid, TRAVERSE_BLOCK, 0, st>>>(S, R, B.shadow[parity], B.film, B.counters,
                                                                         parity);
    }
    else if(S.has_media)
        k_shadow<true><<<grid, TRAVERSE_BLOCK, 0, st>>>(S, R, B.shadow[parity], B.film, B.counters, parity);
    else
        k_shadow<false><<<grid, TRAVERSE_BLOCK, 0, st>>>(S, R, B.shadow[parity], B.film, B.counters, parity);
}

// threads per block of the grid-stride stage kernels (generate, medium, shade); k_order
// is written for BLOCK threads
int stage_block(const DevRender &R) { return R.stage_block > 0 ? R.stage_block : BLOCK; }

// persistent grid of every stage kernel for this scene and render (variants as launched)
void stage_grids(const DevScene &S, const DevRender &R, int grids[6])
{
    const int sb = stage_block(R);
    const bool multi = R.batch != nullptr;
    grids[0] = persistent_grid(sb, multi ? reinterpret_cast<const void *>(k_generate<true>)
                                         : reinterpret_cast<const void *>(k_generate<false>), R.grid_pct);
    grids[1] = persistent_grid(TRAVERSE_BLOCK, multi        ? reinterpret_cast<const void *>(k_trace<false, true>)
                                               : S.two_level ? reinterpret_cast<const void *>(k_trace<false, false, true>)
                                                             : reinterpret_cast<const void *>(k_trace<false>),
                               R.grid_pct);
    grids[2] = persistent_grid(sb, reinterpret_cast<const void *>(k_medium), R.grid_pct);
    grids[3] = persistent_grid(sb, reinterpret_cast<const void *>(shade_kernel(S, R)), R.grid_pct);
    const void *shadow_fn = multi ? reinterpret_cast<const void *>(k_shadow<false, true>)
                            : S.two_level ? (S.has_media ? reinterpret_cast<const void *>(k_shadow<true, false, true>)
                                                         : reinterpret_cast<const void *>(k_shadow<false, false, true>))
                            : S.has_media ? reinterpret_cast<const void *>(k_shadow<true>)
                                          : reinterpret_cast<const void *>(k_shadow<false>);
    grids[4] = persistent_grid(TRAVERSE_BLOCK, shadow_fn, R.grid_pct);
    grids[5] = persistent_grid(BLOCK, reinterpret_cast<const void *>(k_order), R.grid_pct);  // sized for BLOCK
}

// One bounce of the given parity. With defer_shadow the caller launches its shadow kernel
// (on another stream, beside the next bounce).
cudaError_t enqueue_bounce(const DevScene &S, const DevRender &R, RenderBuffers &B, int parity, cudaStream_t st,
                           const int grids[6], int profile, StageTimer *T, uint64_t *launches,
                           bool defer_shadow = false)
{
    PathSoA &P = B.path[parity];
    PathSoA &N = B.path[1 - parity];
    ShadowSoA &SH = B.shadow[parity];
    timed(T, STAGE_CONTROL, st, launches,
          [&] { k_control<<<1, 1, 0, st>>>(B.counters, B.capacity, R.total_paths, parity); });
    timed(T, STAGE_GENERATE, st, launches,
          [&] {
              if(R.batch)
                  k_generate<true><<<grids[0], stage_block(R), 0, st>>>(R, P, B.film, B.counters, S.vacuum_medium);
              else
                  k_generate<false><<<grids[0], stage_block(R), 0, st>>>(R, P, B.film, B.counters, S.vacuum_medium);
          });
    timed(T, STAGE_TRACE, st, launches, [&] {
        if(R.batch)
            k_trace<false, true><<<grids[1], TRAVERSE_BLOCK, 0, st>>>(S, P, B.hit_flag, B.hit_detail, B.counters, R);
        else if(S.two_level)
            k_trace<false, false, true><<<grids[1], TRAVERSE_BLOCK, 0, st>>>(S, P, B.hit_flag, B.hit_detail,
                                                                             B.counters, R);
        else if(profile == 2)
            k_trace<true><<<grids[1], TRAVERSE_BLOCK, 0, st>>>(S, P, B.hit_flag, B.hit_detail, B.counters, R);
        else
            k_trace<false><<<grids[1], TRAVERSE_BLOCK, 0, st>>>(S, P, B.hit_flag, B.hit_detail, B.counters, R);
    });
    if(S.has_media)
        timed(T, STAGE_MEDIUM, st, launches, [&] {
            k_medium<<<grids[2], stage_block(R), 0, st>>>(S, R, P, N, SH, parity, B.hit_flag, B.hit_detail, B.film,
                                                 B.counters);
        });
    timed(T, STAGE_SHADE, st, launches,
          [&] { k_order<<<grids[5], BLOCK, 0, st>>>(B.hit_flag, B.order, B.counters); });
    timed(T, STAGE_SHADE, st, launches, [&] {
        shade_kernel(S, R)<<<grids[3], stage_block(R), 0, st>>>(S, R, P, N, SH, parity, B.hit_flag, B.hit_detail, B.order,
                                                       B.film, B.counters);
    });
    if(!defer_shadow)
        timed(T, STAGE_SHADOW, st, launches, [&] { launch_shadow(S, R, B, parity, st, grids[4]); });
    return cudaGetLastError();
}

} // namespace

cudaError_t upload_primes()
{
    std::vector<uint32_t> primes;
    for(uint32_t v = 2; primes.size() < PRIME_COUNT; ++v)
    {
        bool is_prime = true;
        for(uint32_t p : primes)
        {
            if(p * p > v)
                break;
            if(v % p == 0)
            {
                is_prime = false;
                break;
            }
        }
        if(is_prime)
            primes.push_back(v);
    }
    std::vector<uint64_t> magic(PRIME_COUNT), hash(PRIME_COUNT);
    for(uint32_t d = 0; d < PRIME_COUNT; ++d)
    {
        magic[d] = UINT64_MAX / primes[d] + 1ull;
        hash[d] = mix_bits(static_cast<uint64_t>(1u + (d << 4)));
    }
    cudaError_t e = cudaMemcpyToSymbol(c_primes, primes.data(), sizeof(uint32_t) * PRIME_COUNT);
    if(e == cudaSuccess)
        e = cudaMemcpyToSymbol(c_prime_magic, magic.data(), sizeof(uint64_t) * PRIME_COUNT);
    if(e == cudaSuccess)
        e = cudaMemcpyToSymbol(c_dim_hash, hash.data(), sizeof(uint64_t) * PRIME_COUNT);
    return e;
}

// What render_wavefront keeps with its buffers between calls: the side stream and the
// events of the bounce graph, the instantiated graph (updated in place when only kernel
// arguments change, instantiated anew when the launches differ) and the timing events.
struct RenderGraph
{
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, odd_done = nullptr, even_shaded = nullptr, even_done = nullptr;
    cudaEvent_t ring[RING_SLOTS] = {};
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    cudaGraphExec_t exec = nullptr;
};

void release_render_graph(RenderBuffers &B)
{
    RenderGraph *G = B.graph;
    if(!G)
        return;
    if(G->exec)
        cudaGraphExecDestroy(G->exec);
    for(cudaEvent_t ev : { G->fork, G->odd_done, G->even_shaded, G->even_done, G->t0, G->t1 })
        if(ev)
            cudaEventDestroy(ev);
    for(cudaEvent_t ev : G->ring)
        if(ev)
            cudaEventDestroy(ev);
    if(G->side)
        cudaStreamDestroy(G->side);
    delete G;
    B.graph = nullptr;
}

namespace {

cudaError_t render_graph_setup(RenderBuffers &B)
{
    if(B.graph)
        return cudaSuccess;
    RenderGraph *G = new RenderGraph();
    B.graph = G;
    cudaError_t e = cudaStreamCreateWithFlags(&G->side, cudaStreamNonBlocking);
    for(cudaEvent_t *ev : { &G->fork, &G->odd_done, &G->even_shaded, &G->even_done })
        if(e == cudaSuccess)
            e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    for(cudaEvent_t &ev : G->ring)
        if(e == cudaSuccess)
            e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if(e == cudaSuccess)
        e = cudaEventCreate(&G->t0);
    if(e == cudaSuccess)
        e = cudaEventCreate(&G->t1);
    if(e != cudaSuccess)
        release_render_graph(B);
    return e;
}

} // namespace

cudaError_t render_wavefront(const DevScene &S, const DevRender &R, RenderBuffers &B, cudaStream_t st,
                             const std::atomic<bool> *cancel, bool use_graphs, int profile, RenderStats *stats,
                             bool *cancelled, std::vector<std::pair<double, uint64_t>> *progress,
                             std::vector<uint8_t> *live)
{
    *cancelled = false;
    if(profile != 0)
        use_graphs = false;
    uint64_t launches[STAGE_COUNT] = {};
    uint64_t graph_launches = 0;
    StageTimer timer;
    StageTimer *T = profile == 1 ? &timer : nullptr;
    // every path ends within D + 1 bounces of its generation, and while the queue is full
    // at least `capacity` paths finish every D + 1 bounces: bound the loop so that a
    // malformed configuration cannot spin forever
    const uint64_t depth_bound = static_cast<uint64_t>(std::max(R.max_depth, R.min_depth)) + 2;
    const uint64_t bounce_bound = ((R.total_paths + R.capacity - 1) / R.capacity + 2) * depth_bound;
    const uint64_t max_launches = bounce_bound + RING_SLOTS + 64;  // a launch runs two bounces: 2x slack
    cudaError_t e = cudaMemsetAsync(B.counters, 0, sizeof(Counters), st);
    if(e != cudaSuccess)
        return e;
    int grids[6];
    stage_grids(S, R, grids);

    // Graph of two bounces. Each bounce's shadow kernel runs on a second stream beside the
    // next bounce: the odd bounce's shadow rays are traced at the start of the following
    // launch, beside its even bounce, and once more after the last launch. A bounce that
    // reuses a shadow queue (its control kernel resets the queue's counters) waits for the
    // shadow kernel that reads it.
    if((e = render_graph_setup(B)) != cudaSuccess)
        return e;
    RenderGraph &G = *B.graph;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t side = G.side;
    cudaEvent_t fork = G.fork, odd_done = G.odd_done, even_shaded = G.even_shaded, even_done = G.even_done;
    if(use_graphs)
    {
        e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if(e != cudaSuccess)
            return e;
        uint64_t dummy[STAGE_COUNT] = {};
        cudaEventRecord(fork, st);
        cudaStreamWaitEvent(side, fork, 0);
        launch_shadow(S, R, B, 1, side, grids[4]);
        cudaEventRecord(odd_done, side);
        enqueue_bounce(S, R, B, 0, st, grids, 0, nullptr, dummy, true);
        cudaEventRecord(even_shaded, st);
        cudaStreamWaitEvent(side, even_shaded, 0);
        launch_shadow(S, R, B, 0, side, grids[4]);
        cudaEventRecord(even_done, side);
        cudaStreamWaitEvent(st, odd_done, 0);
        enqueue_bounce(S, R, B, 1, st, grids, 0, nullptr, dummy, true);
        cudaStreamWaitEvent(st, even_done, 0);
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(st, &graph);
        if(e == cudaSuccess)
        {
            // the kept graph takes the new arguments in place when the launches are the
            // same ones; otherwise it is instantiated anew
            if(G.exec)
            {
                cudaGraphExecUpdateResultInfo info{};
                if(cudaGraphExecUpdate(G.exec, graph, &info) != cudaSuccess)
                {
                    cudaGetLastError();
                    cudaGraphExecDestroy(G.exec);
                    G.exec = nullptr;
                }
            }
            if(!G.exec)
                e = cudaGraphInstantiate(&G.exec, graph, 0);
            cudaGraphDestroy(graph);
        }
        if(e != cudaSuccess)
        {
            if(G.exec)
                cudaGraphExecDestroy(G.exec);
            G.exec = nullptr;
            return e;
        }
        exec = G.exec;
    }

    cudaEvent_t *ev = G.ring;
    cudaEvent_t t0 = G.t0, t1 = G.t1;
    // progress log: one timing event and one copy of the generated-path counter per launch
    std::vector<cudaEvent_t> prog_ev;
    uint64_t *prog_gen = nullptr;
    uint8_t *prog_live = nullptr;
    const size_t live_stride = R.batch ? R.batch_count : 0;
    if(progress && use_graphs)
    {
        progress->clear();
        if(cudaMalloc(&prog_gen, sizeof(uint64_t) * (max_launches + 1)) != cudaSuccess)
        {
            prog_gen = nullptr;
            cudaGetLastError();
        }
        if(prog_gen && live && live_stride)
        {
            if(cudaMalloc(&prog_live, live_stride * (max_launches + 1)) != cudaSuccess ||
               cudaMemsetAsync(prog_live, 0, live_stride * (max_launches + 1), st) != cudaSuccess)
            {
                cudaFree(prog_live);
                prog_live = nullptr;
                cudaGetLastError();
            }
        }
    }
    cudaEventRecord(t0, st);

    // Launch pairs of bounces; read the counters back asynchronously and test completion
    // RING_SLOTS-1 launches behind, so the GPU never idles waiting for the host.
    uint64_t launches_total = 0;
    for(;;)
    {
        const uint64_t launches_now = launches_total;
        const int slot = static_cast<int>(launches_now % RING_SLOTS);
        if(launches_now >= RING_SLOTS - 1)
        {
            const int old = static_cast<int>((launches_now - (RING_SLOTS - 1)) % RING_SLOTS);
            e = cudaEventSynchronize(ev[old]);
            if(e != cudaSuccess)
                break;
            const Counters &c = B.host_counters[old];
            if(c.generated >= R.total_paths && c.next_active == 0)
                break;
            if(cancel && cancel->load())
            {
                *cancelled = true;
                break;
            }
        }
        if(launches_now >= max_launches)
        {
            e = cudaErrorLaunchTimeout;
            break;
        }
        if(use_graphs)
        {
            e = cudaGraphLaunch(exec, st);
            ++graph_launches;
        }
        else
        {
            e = enqueue_bounce(S, R, B, 0, st, grids, profile, T, launches_by_stage_ptr(launches));
            if(e == cudaSuccess)
                e = enqueue_bounce(S, R, B, 1, st, grids, profile, T, launches_by_stage_ptr(launches));
        }
        if(e != cudaSuccess)
            break;
        if(prog_gen)
        {
            cudaEvent_t pe;
            cudaEventCreate(&pe);
            cudaEventRecord(pe, st);
            prog_ev.push_back(pe);
            cudaMemcpyAsync(prog_gen + launches_now, &B.counters->generated, sizeof(uint64_t), cudaMemcpyDeviceToDevice,
                            st);
            // survivors of the launch's second (odd) bounce sit in queue 0
            if(prog_live)
                k_batch_live<<<persistent_grid(BLOCK, reinterpret_cast<const void *>(k_batch_live), 100), BLOCK, 0,
                               st>>>(R, B.path[0].rad_pixel, B.counters, prog_live + launches_now * live_stride);
        }
        cudaMemcpyAsync(&B.host_counters[slot], B.counters, sizeof(Counters), cudaMemcpyDeviceToHost, st);
        cudaEventRecord(ev[slot], st);
        ++launches_total;
    }
    // the last launch's odd-bounce shadow rays
    if(use_graphs && e == cudaSuccess)
    {
        launch_shadow(S, R, B, 1, st, grids[4]);
        e = cudaGetLastError();
    }
    cudaEventRecord(t1, st);
    cudaError_t se = cudaEventSynchronize(t1);
    if(e == cudaSuccess)
        e = se;
    float ms = 0;
    cudaEventElapsedTime(&ms, t0, t1);
    if(prog_gen)
    {
        std::vector<uint64_t> gen(prog_ev.size());
        if(!gen.empty())
            cudaMemcpy(gen.data(), prog_gen, sizeof(uint64_t) * gen.size(), cudaMemcpyDeviceToHost);
        for(size_t k = 0; k < prog_ev.size(); ++k)
        {
            float t = 0;
            cudaEventElapsedTime(&t, t0, prog_ev[k]);
            progress->emplace_back(t, gen[k]);
            cudaEventDestroy(prog_ev[k]);
        }
        cudaFree(prog_gen);
        if(prog_live)
        {
            live->assign(live_stride * prog_ev.size(), 1);
            if(!prog_ev.empty())
                cudaMemcpy(live->data(), prog_live, live_stride * prog_ev.size(), cudaMemcpyDeviceToHost);
            cudaFree(prog_live);
        }
    }
    Counters fin{};
    cudaMemcpy(&fin, B.counters, sizeof(Counters), cudaMemcpyDeviceToHost);
    if(stats)
    {
        *stats = RenderStats{};
        stats->paths = fin.generated;
        stats->ext_rays = fin.ext_rays;
        stats->shadow_rays = fin.shadow_rays + fin.shadow_n[0] + fin.shadow_n[1];
        stats->iterations = fin.iterations;
        stats->err = fin.err;
        stats->device_ms = ms;
        stats->node_visits = fin.node_visits;
        stats->tri_tests = fin.tri_tests;
        // per bounce: control, generate, trace, [medium], order + shade, shadow
        const uint64_t per_bounce = S.has_media ? 7 : 6;
        for(int k = 0; k < STAGE_COUNT; ++k)
            stats->stage_launches[k] = launches[k];
        if(use_graphs)
        {
            for(int k = 0; k < STAGE_COUNT; ++k)
                stats->stage_launches[k] = (k == STAGE_MEDIUM && !S.has_media) ? 0
                                           : k == STAGE_SHADE                    ? graph_launches * 4
                                           : k == STAGE_SHADOW                   ? graph_launches * 2 + 1
                                                                                 : graph_launches * 2;
            stats->kernel_launches = graph_launches * 2 * per_bounce + 1;
        }
        else
        {
            uint64_t total = 0;
            for(int k = 0; k < STAGE_COUNT; ++k)
                total += launches[k];
            stats->kernel_launches = total;
        }
        for(auto &m : timer.marks)
        {
            float t = 0;
            cudaEventElapsedTime(&t, m.second.first, m.second.second);
            stats->stage_ms[m.first] += t;
        }
    }
    return e;
}

// preview kernels for the g-buffer (wavefront/preview.cpp:27-78): sum / weight, and
// normals renormalised (zero when shorter than 1e-3)
__global__ void k_resolve_aov(const float4 *film, const float4 *aov, float *out, uint32_t pixels, int normal)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= pixels)
        return;
    const float w = film[i].w;
    const float4 v = aov[i];
    V3 o(0.0f);
    if(w > 0)
    {
        o = V3(v.x, v.y, v.z) / w;
        if(normal)
            o = length(o) > 1e-3f ? normalize(o) : V3(0.0f);
    }
    out[i * 3 + 0] = o.x;
    out[i * 3 + 1] = o.y;
    out[i * 3 + 2] = o.z;
}

// ACESToneMap (builtin/btrc/builtin/postprocess/tonemap.cpp:14-53): the ACES filmic fit
// x (2.51 x + 0.03) / (x (2.43 x + 0.59) + 0.14), saturated, on exposure-scaled RGB
__device__ __forceinline__ float aces(float x)
{
    const float v = (x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f);
    return fminf(fmaxf(v, 0.0f), 1.0f);
}

__global__ void k_tonemap_aces(float *px, uint32_t pixels, int channels, float exposure)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= pixels)
        return;
    float *p = px + static_cast<size_t>(i) * channels;
    p[0] = aces(p[0] * exposure);
    p[1] = aces(p[1] * exposure);
    p[2] = aces(p[2] * exposure);
}

cudaError_t launch_resolve_aov(const float4 *film, const float4 *aov, float *out, uint32_t pixels, bool normal,
                               cudaStream_t st)
{
    if(pixels == 0)
        return cudaSuccess;
    k_resolve_aov<<<(pixels + 255) / 256, 256, 0, st>>>(film, aov, out, pixels, normal ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_tonemap_aces(float *px, uint32_t pixels, int channels, float exposure, cudaStream_t st)
{
    if(pixels == 0)
        return cudaSuccess;
    k_tonemap_aces<<<(pixels + 255) / 256, 256, 0, st>>>(px, pixels, channels, exposure);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- denoise post-processor

// Edge-avoiding a-trous wavelet filter (Dammertz, Sewtz, Hanika and Lensch, "Edge-Avoiding
// A-Trous Wavelet Transform for fast Global Illumination Filtering", HPG 2010), the stand-in
// for the reference's `denoise` post-processor, whose OptiX AI denoiser is a closed library
// (builtin/btrc/builtin/postprocess/optix_denoiser.cpp:51-126: in place on the colour, with
// optional albedo and normal guides). Pass k convolves with the 5x5 B3-spline kernel
// (1/16, 1/4, 3/8, 1/4, 1/16) dilated to a tap spacing of 2^k pixels; each tap is weighted
// by exp(-(e_c + e_a + e_n)) with e_c = |T(c_p) - T(c_q)|^2 / sigma_c^2, T(c) = c / (1 + c)
// per channel (HDR colours compared in a bounded space) and sigma_c halved every pass,
// e_a = |a_p - a_q|^2 / sigma_a^2 and e_n = |n_p - n_q|^2 / (4^k sigma_n^2) when the guides
// are present. Taps outside the image are skipped and the weights renormalised.
namespace
{
__device__ __forceinline__ float3 ld3(const float *__restrict__ a, size_t i)
{
    return make_float3(a[i * 3 + 0], a[i * 3 + 1], a[i * 3 + 2]);
}

__device__ __forceinline__ float3 tone01(float3 c)
{
    c.x = fmaxf(c.x, 0.0f);
    c.y = fmaxf(c.y, 0.0f);
    c.z = fmaxf(c.z, 0.0f);
    return make_float3(c.x / (1.0f + c.x), c.y / (1.0f + c.y), c.z / (1.0f + c.z));
}

__device__ __forceinline__ float dist2(float3 a, float3 b)
{
    const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return dx * dx + dy * dy + dz * dz;
}
} // namespace

__global__ void __launch_bounds__(256) k_denoise_atrous(const float *__restrict__ in, float *__restrict__ out,
                                                        const float *__restrict__ alb, const float *__restrict__ nrm,
                                                        int w, int h, int step, float inv_sc2, float inv_sa2,
                                                        float inv_sn2)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if(x >= w || y >= h)
        return;
    const size_t p = static_cast<size_t>(y) * w + x;
    const float3 tp = tone01(ld3(in, p));
    const float3 ap = alb ? ld3(alb, p) : make_float3(0.0f, 0.0f, 0.0f);
    const float3 np = nrm ? ld3(nrm, p) : make_float3(0.0f, 0.0f, 0.0f);
    const float hk[3] = { 0.375f, 0.25f, 0.0625f };
    float sx = 0.0f, sy = 0.0f, sz = 0.0f, sw = 0.0f;
    for(int dy = -2; dy <= 2; ++dy)
    {
        const int qy = y + dy * step;
        if(qy < 0 || qy >= h)
            continue;
        for(int dx = -2; dx <= 2; ++dx)
        {
            const int qx = x + dx * step;
            if(qx < 0 || qx >= w)
                continue;
            const size_t q = static_cast<size_t>(qy) * w + qx;
            const float3 cq = ld3(in, q);
            float e = dist2(tp, tone01(cq)) * inv_sc2;
            if(alb)
                e += dist2(ap, ld3(alb, q)) * inv_sa2;
            if(nrm)
                e += dist2(np, ld3(nrm, q)) * inv_sn2;
            const float wt = hk[dx < 0 ? -dx : dx] * hk[dy < 0 ? -dy : dy] * expf(-e);
            sx += wt * cq.x;
            sy += wt * cq.y;
            sz += wt * cq.z;
            sw += wt;
        }
    }
    // the centre tap (weight 9/64) is always present, so sw > 0
    out[p * 3 + 0] = sx / sw;
    out[p * 3 + 1] = sy / sw;
    out[p * 3 + 2] = sz / sw;
}

cudaError_t launch_denoise_atrous(float *rgb, float *tmp, const float *albedo, const float *normal, int width,
                                  int height, cudaStream_t st)
{
    if(width <= 0 || height <= 0)
        return cudaSuccess;
    const dim3 block(16, 16), grid((width + 15) / 16, (height + 15) / 16);
    float *src = rgb, *dst = tmp;
    for(int k = 0; k < DENOISE_PASSES; ++k)
    {
        const float step = static_cast<float>(1 << k);
        const float sc = DENOISE_SIGMA_COLOR / step;  // halved every pass
        k_denoise_atrous<<<grid, block, 0, st>>>(src, dst, albedo, normal, width, height, 1 << k, 1.0f / (sc * sc),
                                                 1.0f / (DENOISE_SIGMA_ALBEDO * DENOISE_SIGMA_ALBEDO),
                                                 1.0f / (DENOISE_SIGMA_NORMAL * DENOISE_SIGMA_NORMAL * step * step));
        std::swap(src, dst);
    }
    if(src != rgb)
        return cudaMemcpyAsync(rgb, src, sizeof(float) * 3 * static_cast<size_t>(width) * height,
                               cudaMemcpyDeviceToDevice, st);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- radiance-cache training paths

constexpr int NRC_TRAIN_VERTS = 6;   // recorded vertices per training path

// Training paths for the radiance cache: one thread traces one whole path of a training
// pixel with the wavefront's per-path semantics (same light sampling, MIS, Russian
// roulette and BSDF sampling; the shadow ray is traced at once), records its first
// non-delta vertices (cache query, throughput, radiance gathered so far) and, when the
// path ends, emits one sample per vertex whose target is the radiance the path gathered
// after that vertex divided by the throughput at it: an unbiased estimate of the
// vertex's outgoing radiance. Scenes with participating media are not supported here.
template<bool TEX>
__global__ void __launch_bounds__(128) k_nrc_train_paths(DevScene S, DevRender R, uint32_t stride, uint32_t phase,
                                                         uint32_t sample_index, float *samples, uint32_t *count,
                                                         uint32_t cap, uint32_t *err)
{
    const uint32_t pixels = static_cast<uint32_t>(R.width) * R.height;
    const uint32_t n = phase < pixels ? (pixels - phase + stride - 1) / stride : 0;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const uint32_t pixel = i * stride + phase;
        const uint32_t px = pixel % R.width, py = pixel / R.width;
        DSampler smp;
        smp.type = R.sampler;
        smp.s = sampler_init(R.sampler, R.halton, px, py, sample_index);
        float fx, fy;
        if(R.filter == FILTER_GAUSSIAN)
        {
            const uint32_t cell = alias_sample(R.filter_table, FILTER_GRID * FILTER_GRID, smp.get1d());
            const uint32_t gy = cell / FILTER_GRID, gx = cell % FILTER_GRID;
            const float r = R.filter_radius, w = 2 * r / FILTER_GRID;
            fx = lerpf(-r + w * static_cast<float>(gx), -r + w * static_cast<float>(gx + 1), smp.get1d());
            fy = lerpf(-r + w * static_cast<float>(gy), -r + w * static_cast<float>(gy + 1), smp.get1d());
        }
        else
        {
            fx = smp.get1d() - 0.5f;
            fy = smp.get1d() - 0.5f;
        }
        (void)smp.get1d();
        const float film_x = (static_cast<float>(px) + 0.5f + fx) / static_cast<float>(R.width);
        const float film_y = (static_cast<float>(py) + 0.5f + fy) / static_cast<float>(R.height);
        V3 o = R.cam_eye;
        V3 d = normalize(R.cam_lbc + film_x * R.cam_fx + film_y * R.cam_fy - R.cam_eye);
        V3 beta(1.0f), beta_le(1.0f), rad(0.0f);
        float bsdf_pdf = -1.0f;
        float vq[NRC_TRAIN_VERTS][NRC_QUERY_FLOATS];
        V3 vbeta[NRC_TRAIN_VERTS], vrad[NRC_TRAIN_VERTS];
        int nv = 0;
        for(int depth = 0; depth < 256; ++depth)
        {
            const float ro3[3] = { o.x, o.y, o.z }, rd3[3] = { d.x, d.y, d.z };
            const ClosestResult c = scene_closest(S, ro3, rd3, MAX_FLOAT, err);
            if(!c.hit)
            {
                rad = rad + miss_le(S, d, beta_le, bsdf_pdf);
                break;
            }
            const Instance &inst = S.instances[c.inst];
            const Geometry geo = S.geometries[inst.geometry];
            const SurfacePoint sp = get_hitinfo(S, o, d, inst, geo.tri_offset + c.prim, c.t, c.b1, c.b2);
            rad = rad + hit_light_le(S, o, d, sp, beta_le, bsdf_pdf, inst.light);
            if(nv < NRC_TRAIN_VERTS && nrc_query_at<TEX>(S, sp, inst, -d, vq[nv]))
            {
                vbeta[nv] = beta;
                vrad[nv] = rad;
                ++nv;
            }
            if(russian_roulette(beta, depth, smp, R))
                break;
            LightSample ls = sample_light(S, sp.position, sp.frame.z, true, smp);
            Material mat = S.materials[inst.material];
            SurfaceShader sh;
            sh.frame.geometry = sp.frame;
            sh.frame.shading = sp.frame.rotate_to_new_z(sp.interp_z);
            if(TEX && mat.tex >= 0)
            {
                const MaterialTexValues tv = eval_material_textures(S, mat.tex, sp.tu, sp.tv);
#pragma unroll
                for(int k = 0; k < 16; ++k)
                    if(tv.mask & (1u << k))
                        mat.p[k] = tv.p[k];
                if(tv.has_normal)
                    sh.frame.shading =
                        sh.frame.shading.rotate_to_new_z(normalize(sh.frame.shading.local_to_global(tv.normal)));
            }
            sh.mat = make_material_eval(mat);
            sh.shadow_terminator = mat.shadow_terminator != 0;
            float u0, u1, u2;
            smp.get3d(u0, u1, u2);
            const V3 wo = -d;
            V3 f;
            float spdf;
            const CompSample bs = sh.sample_eval(wo, u0, u1, u2, ls.success, ls.d, f, spdf);
            if(ls.success)
            {
                if(!is_zero(f))
                {
                    const float cs = fabsf(dot(normalize(ls.d), sp.frame.z));
                    const V3 li = ls.li * beta * f * cs / (spdf + ls.light_pdf);
                    const float so3[3] = { ls.o.x, ls.o.y, ls.o.z }, sd3[3] = { ls.d.x, ls.d.y, ls.d.z };
                    if(!scene_any(S, so3, sd3, ls.t1, err) && all_finite(li))
                        rad = rad + li;
                }
            }
            if(is_zero(bs.f))
                break;
            const V3 ndir = normalize(bs.dir);
            const float cn = fabsf(dot(ndir, sp.frame.z));
            beta_le = beta * cn * bs.f;
            beta = beta_le / bs.pdf;
            bsdf_pdf = bs.is_delta ? -bs.pdf : bs.pdf;
            o = offset_dir(sp.position, sp.frame.z, ndir);
            d = ndir;
        }
        for(int k = 0; k < nv; ++k)
        {
            const V3 b = vbeta[k];
            if(!(b.x > 1e-6f && b.y > 1e-6f && b.z > 1e-6f))
                continue;
            const V3 t = (rad - vrad[k]) / b;
            if(!all_finite(t))
                continue;
            const uint32_t slot = atomicAdd(count, 1u);
            if(slot >= cap)
                break;
            float *dst = samples + static_cast<size_t>(slot) * NRC_SAMPLE_FLOATS;
            for(int j = 0; j < NRC_QUERY_FLOATS; ++j)
                dst[j] = vq[k][j];
            dst[13] = fmaxf(t.x, 0.0f);
            dst[14] = fmaxf(t.y, 0.0f);
            dst[15] = fmaxf(t.z, 0.0f);
        }
    }
}

// cache predictions times path throughput, splatted to the paths' pixels
__global__ void k_nrc_splat(const float4 *__restrict__ pred, const float4 *__restrict__ weight, const uint32_t *count,
                            uint32_t cap, float4 *film, int width)
{
    const uint32_t n = min(*count, cap);
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const float4 p = pred[i], w = weight[i];
        splat(film, __float_as_uint(w.w), width, V3(fmaxf(p.x, 0.0f) * w.x, fmaxf(p.y, 0.0f) * w.y, fmaxf(p.z, 0.0f) * w.z));
    }
}

cudaError_t launch_nrc_train_paths(const DevScene &S, const DevRender &R, uint32_t stride, uint32_t phase,
                                   uint32_t sample_index, float *samples, uint32_t *count, uint32_t cap, uint32_t *err,
                                   cudaStream_t st)
{
    const uint32_t pixels = static_cast<uint32_t>(R.width) * R.height;
    const uint32_t n = phase < pixels ? (pixels - phase + stride - 1) / stride : 0;
    if(n == 0)
        return cudaSuccess;
    const uint32_t blocks = (n + 127) / 128;
    if(S.material_tex != nullptr)
        k_nrc_train_paths<true><<<blocks, 128, 0, st>>>(S, R, stride, phase, sample_index, samples, count, cap, err);
    else
        k_nrc_train_paths<false><<<blocks, 128, 0, st>>>(S, R, stride, phase, sample_index, samples, count, cap, err);
    return cudaGetLastError();
}

cudaError_t launch_nrc_splat(const float4 *pred, const float4 *weight, const uint32_t *count, uint32_t cap,
                             float4 *film, int width, cudaStream_t st)
{
    if(cap == 0)
        return cudaSuccess;
    k_nrc_splat<<<std::min<uint32_t>((cap + 255) / 256, 152 * 16), 256, 0, st>>>(pred, weight, count, cap, film, width);
    return cudaGetLastError();
}

cudaError_t launch_resolve(const float4 *film, float *rgb, uint32_t pixels, cudaStream_t st)
{
    if(pixels == 0)
        return cudaSuccess;
    k_resolve<<<(pixels + 255) / 256, 256, 0, st>>>(film, rgb, pixels);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- merged batches
//
// Several built scenes concatenated into one device scene: node, triangle, instance,
// geometry, material, light and medium arrays placed one scene after another, with every
// index a record holds shifted by its scene's offsets (applied by the kernels below to
// each scene's slice after the copy).

namespace {

__global__ void k_rebase_scene(CWNode *nodes, uint32_t n_nodes, TriRec *tris, uint32_t n_tris, Instance *inst,
                               uint32_t n_inst, Geometry *geo, uint32_t n_geo, AreaLight *lights, uint32_t n_lights,
                               RebaseOffsets o)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_nodes; i += stride)
    {
        nodes[i].child_base += o.node;
        nodes[i].tri_base += o.tri;
    }
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_tris; i += stride)
        tris[i].inst += o.inst;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_inst; i += stride)
    {
        Instance &x = inst[i];
        x.geometry += static_cast<int32_t>(o.geo);
        x.material += static_cast<int32_t>(o.mat);
        // x.light stays an index into its own scene's lights: the merged kernels read the
        // scene's light table through a view that starts at the scene's first light
        const uint32_t inner = (x.media & 0xffffu) + o.med, outer = (x.media >> 16) + o.med;
        x.media = (inner & 0xffffu) | (outer << 16);
    }
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_geo; i += stride)
    {
        Geometry &g = geo[i];
        g.tri_offset += o.shade_tri;
        uint32_t lo;
        memcpy(&lo, &g.pad, sizeof(lo));
        if(lo != 0xffffffffu)
        {
            lo += o.light_tri;
            memcpy(&g.pad, &lo, sizeof(lo));
        }
    }
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_lights; i += stride)
    {
        lights[i].instance += static_cast<int32_t>(o.inst);
        lights[i].geometry += static_cast<int32_t>(o.geo);
    }
}

// radiance / weight of each scene's band of the combined film into its own image
__global__ void k_resolve_batch(const float4 *film, uint32_t film_width, const BatchOut *outs)
{
    const BatchOut o = outs[blockIdx.y];
    const uint32_t pixels = o.width * o.height;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < pixels; i += gridDim.x * blockDim.x)
    {
        const uint32_t x = i % o.width, y = i / o.width;
        const float4 f = film[static_cast<size_t>(o.row_base + y) * film_width + x];
        const float inv = f.w > 0 ? 1.0f / f.w : 0.0f;
        o.rgb[static_cast<size_t>(i) * 3 + 0] = f.x * inv;
        o.rgb[static_cast<size_t>(i) * 3 + 1] = f.y * inv;
        o.rgb[static_cast<size_t>(i) * 3 + 2] = f.z * inv;
    }
}

} // namespace

cudaError_t launch_rebase_scene(CWNode *nodes, uint32_t n_nodes, TriRec *tris, uint32_t n_tris, Instance *inst,
                                uint32_t n_inst, Geometry *geo, uint32_t n_geo, AreaLight *lights, uint32_t n_lights,
                                const RebaseOffsets &o, cudaStream_t st)
{
    const uint32_t n = std::max(std::max(n_nodes, n_tris), std::max(n_inst, std::max(n_geo, n_lights)));
    if(n == 0)
        return cudaSuccess;
    const uint32_t blocks = std::min<uint32_t>((n + 255) / 256, 4096);
    k_rebase_scene<<<blocks, 256, 0, st>>>(nodes, n_nodes, tris, n_tris, inst, n_inst, geo, n_geo, lights, n_lights, o);
    return cudaGetLastError();
}

cudaError_t launch_resolve_batch(const float4 *film, uint32_t film_width, const BatchOut *outs, uint32_t count,
                                 uint32_t max_pixels, cudaStream_t st)
{
    if(count == 0)
        return cudaSuccess;
    const uint32_t bx = std::min<uint32_t>((max_pixels + 255) / 256, 1024);
    k_resolve_batch<<<dim3(bx, count), 256, 0, st>>>(film, film_width, outs);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- allocation-free render
//
// For callers that cannot allocate GPU memory while they render: engines that reserve
// all device memory up front and hand out nothing afterwards, processes running under a
// hard memory budget, or code that must not call cudaMalloc/cudaFree (which synchronise
// the device) on a latency-critical thread. Everything the wavefront loop needs beyond
// the scene and the caller's output image lives in one fixed array below, reserved when
// the library's kernels are loaded on a device and kept until the process exits.

namespace {

constexpr uint32_t NOALLOC_MAX_STATES = 32768;   // path-queue capacity
constexpr uint32_t NOALLOC_MAX_PIXELS = 512 * 512;
constexpr size_t NOALLOC_PATH_BYTES = 6 * 16;    // one PathSoA slot
constexpr size_t NOALLOC_BYTES =
    2 * NOALLOC_PATH_BYTES * NOALLOC_MAX_STATES      // current + next queues
    + 2 * 4 * 16 * NOALLOC_MAX_STATES                 // two shadow queues (o, d, beta, sampler)
    + (4 + 16 + 4) * NOALLOC_MAX_STATES               // hit flags + details + shade order
    + 16 * static_cast<size_t>(NOALLOC_MAX_PIXELS)    // film
    + 256                                             // counters
    + 40 * 256;                                       // 256-byte alignment of each buffer

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
void *g_noalloc_addr[NOALLOC_MAX_DEVICES] = {};
int g_noalloc_contexts[NOALLOC_MAX_DEVICES] = {};   // live btrc contexts per device

} // namespace

size_t noalloc_scratch_bytes() { return NOALLOC_BYTES; }
uint32_t noalloc_max_states() { return NOALLOC_MAX_STATES; }
uint32_t noalloc_max_pixels() { return NOALLOC_MAX_PIXELS; }

// Device address of the scratch array for the current device. The host-side name of a
// __device__ variable is only a stand-in, so the address is looked up once per device
// (with that device current) and cached while a context of this library is alive on that
// device; when the last one is destroyed the entry is dropped, so a device reset between
// contexts (which reloads the module and moves the array) cannot leave a stale address.
void noalloc_context_opened(int device)
{
    if(device < 0 || device >= NOALLOC_MAX_DEVICES)
        return;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    ++g_noalloc_contexts[device];
}

void noalloc_context_closed(int device)
{
    if(device < 0 || device >= NOALLOC_MAX_DEVICES)
        return;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if(g_noalloc_contexts[device] > 0 && --g_noalloc_contexts[device] == 0)
        g_noalloc_addr[device] = nullptr;
}

cudaError_t noalloc_scratch_address(int device, void **out)
{
    if(device < 0 || device >= NOALLOC_MAX_DEVICES)
        return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if(!g_noalloc_addr[device])
    {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if(e != cudaSuccess)
            return e;
        g_noalloc_addr[device] = ptr;
    }
    *out = g_noalloc_addr[device];
    return cudaSuccess;
}

cudaError_t render_wavefront_noalloc(const DevScene &S, const DevRender &R, void *scratch, float *rgb_out,
                                     cudaStream_t st, const std::atomic<bool> *cancel, RenderStats *stats,
                                     bool *cancelled)
{
    *cancelled = false;
    const uint32_t cap = R.capacity;
    const size_t pixels = static_cast<size_t>(R.width) * R.height;
    // carve the fixed array into the same buffers render_wavefront uses
    unsigned char *p = static_cast<unsigned char *>(scratch);
    auto take = [&](size_t bytes) {
        unsigned char *r = p;
        p += (bytes + 255) / 256 * 256;
        return r;
    };
    RenderBuffers B{};
    for(int k = 0; k < 2; ++k)
    {
        B.path[k].beta_depth = reinterpret_cast<F4 *>(take(16ull * cap));
        B.path[k].rad_pixel = reinterpret_cast<F4 *>(take(16ull * cap));
        B.path[k].sampler = reinterpret_cast<SamplerState *>(take(16ull * cap));
        B.path[k].ray_o = reinterpret_cast<F4 *>(take(16ull * cap));
        B.path[k].ray_d = reinterpret_cast<F4 *>(take(16ull * cap));
        B.path[k].bsdf_le = reinterpret_cast<F4 *>(take(16ull * cap));
    }
    for(int k = 0; k < 2; ++k)
    {
        B.shadow[k].o = reinterpret_cast<F4 *>(take(16ull * cap));
        B.shadow[k].d = reinterpret_cast<F4 *>(take(16ull * cap));
        B.shadow[k].beta = reinterpret_cast<F4 *>(take(16ull * cap));
        B.shadow[k].sampler = reinterpret_cast<SamplerState *>(take(16ull * cap));
    }
    B.hit_flag = reinterpret_cast<uint32_t *>(take(4ull * cap));
    B.hit_detail = reinterpret_cast<HitDetail *>(take(16ull * cap));
    B.order = reinterpret_cast<uint32_t *>(take(4ull * cap));
    B.film = reinterpret_cast<float4 *>(take(16ull * pixels));
    B.counters = reinterpret_cast<Counters *>(take(sizeof(Counters)));
    B.host_counters = nullptr;
    B.capacity = cap;
    if(static_cast<size_t>(p - static_cast<unsigned char *>(scratch)) > NOALLOC_BYTES)
        return cudaErrorInvalidValue;

    // the array keeps the previous call's contents: clear the film and the counters
    cudaError_t e = cudaMemsetAsync(B.film, 0, 16ull * pixels, st);
    if(e == cudaSuccess)
        e = cudaMemsetAsync(B.counters, 0, sizeof(Counters), st);
    if(e != cudaSuccess)
        return e;
    int grids[6];
    stage_grids(S, R, grids);
    const uint64_t depth_bound = static_cast<uint64_t>(std::max(R.max_depth, R.min_depth)) + 2;
    const uint64_t max_launches = ((R.total_paths + cap - 1) / cap + 2) * depth_bound + 64;
    uint64_t launches[STAGE_COUNT] = {};
    Counters c{};
    for(uint64_t launch = 0;; ++launch)
    {
        if(launch >= max_launches)
        {
            e = cudaErrorLaunchTimeout;
            break;
        }
        e = enqueue_bounce(S, R, B, 0, st, grids, 0, nullptr, launches);
        if(e == cudaSuccess)
            e = enqueue_bounce(S, R, B, 1, st, grids, 0, nullptr, launches);
        // counters come back synchronously into this stack variable: no pinned buffer
        if(e == cudaSuccess)
            e = cudaMemcpyAsync(&c, B.counters, sizeof(Counters), cudaMemcpyDeviceToHost, st);
        if(e == cudaSuccess)
            e = cudaStreamSynchronize(st);
        if(e != cudaSuccess)
            break;
        if(c.generated >= R.total_paths && c.next_active == 0)
            break;
        if(cancel && cancel->load())
        {
            *cancelled = true;
            break;
        }
    }
    if(e == cudaSuccess)
        e = launch_resolve(B.film, rgb_out, static_cast<uint32_t>(pixels), st);
    if(e == cudaSuccess)
        e = cudaMemcpyAsync(&c, B.counters, sizeof(Counters), cudaMemcpyDeviceToHost, st);
    if(e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if(stats)
    {
        *stats = RenderStats{};
        stats->paths = c.generated;
        stats->ext_rays = c.ext_rays;
        stats->shadow_rays = c.shadow_rays + c.shadow_n[0] + c.shadow_n[1];
        stats->iterations = c.iterations;
        stats->err = c.err;
        uint64_t total = 0;
        for(int k = 0; k < STAGE_COUNT; ++k)
        {
            stats->stage_launches[k] = launches[k];
            total += launches[k];
        }
        stats->kernel_launches = total + 1;
    }
    return e;
}

// ---------------------------------------------------------------- test hooks

namespace {

__global__ void k_sampler_batch(int type, int width, int height, HaltonConsts hc, const uint32_t *pix,
                                const uint32_t *sidx, uint32_t n, uint32_t dims, float *out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n)
        return;
    (void)width;
    (void)height;
    DSampler smp;
    smp.type = type;
    const uint32_t p = pix[i];
    smp.s = sampler_init(type, hc, p & 0xffffu, p >> 16, sidx[i]);
    for(uint32_t k = 0; k < dims; ++k)
        out[static_cast<size_t>(i) * dims + k] = smp.get1d();
}

__global__ void k_bsdf_batch(int op, const Material *mats, const float *wo, const float *wu, uint32_t n, float *out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n)
        return;
    Material m = mats[i];
    const V3 lwo(wo[i * 3 + 0], wo[i * 3 + 1], wo[i * 3 + 2]);
    const MaterialEval e = make_material_eval(m);
    if(op == 0)
    {
        const V3 lwi(wu[i * 3 + 0], wu[i * 3 + 1], wu[i * 3 + 2]);
        V3 f;
        float pdf;
        comp_eval_pdf(e, lwi, lwo, f, pdf);
        out[i * 4 + 0] = f.x;
        out[i * 4 + 1] = f.y;
        out[i * 4 + 2] = f.z;
        out[i * 4 + 3] = pdf;
    }
    else if(op == 2)
    {
        // the sampled direction alone, before Disney's bad-sample rejection
        V3 lwi(0.0f);
        const bool ok = comp_sample_dir(e, lwo, wu[i * 3 + 0], wu[i * 3 + 1], wu[i * 3 + 2], lwi);
        out[i * 7 + 0] = ok ? 1.0f : 0.0f;
        out[i * 7 + 1] = 0.0f;
        out[i * 7 + 2] = 0.0f;
        out[i * 7 + 3] = 0.0f;
        out[i * 7 + 4] = ok ? lwi.x : 0.0f;
        out[i * 7 + 5] = ok ? lwi.y : 0.0f;
        out[i * 7 + 6] = ok ? lwi.z : 0.0f;
    }
    else
    {
        const CompSample s = comp_sample(e, lwo, wu[i * 3 + 0], wu[i * 3 + 1], wu[i * 3 + 2]);
        out[i * 7 + 0] = s.f.x;
        out[i * 7 + 1] = s.f.y;
        out[i * 7 + 2] = s.f.z;
        out[i * 7 + 3] = s.pdf;
        out[i * 7 + 4] = s.dir.x;
        out[i * 7 + 5] = s.dir.y;
        out[i * 7 + 6] = s.dir.z;
    }
}

__global__ void k_medium_tr_batch(DevScene S, int medium_id, const float *seg, const uint64_t *seeds, uint32_t n,
                                  float *out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n)
        return;
    DSampler smp;
    smp.type = SAMPLER_INDEPENDENT;
    pcg32_seed(smp.s.a, smp.s.b, seeds[i], PCG_STREAM);
    const V3 a(seg[i * 6 + 0], seg[i * 6 + 1], seg[i * 6 + 2]);
    const V3 b(seg[i * 6 + 3], seg[i * 6 + 4], seg[i * 6 + 5]);
    out[i] = medium_tr(S, S.media[medium_id], a, b, smp).x;
}

} // namespace

cudaError_t launch_sampler_batch(int type, int width, int height, const HaltonConsts &hc, const uint32_t *pixel_xy,
                                 const uint32_t *sample_index, uint32_t n, uint32_t dims, float *out, cudaStream_t st)
{
    if(n == 0)
        return cudaSuccess;
    k_sampler_batch<<<(n + 127) / 128, 128, 0, st>>>(type, width, height, hc, pixel_xy, sample_index, n, dims, out);
    return cudaGetLastError();
}

cudaError_t launch_bsdf_batch(int op, const Material *mats, const float *wo, const float *wi_or_u, uint32_t n,
                              float *out, cudaStream_t st)
{
    if(n == 0)
        return cudaSuccess;
    k_bsdf_batch<<<(n + 127) / 128, 128, 0, st>>>(op, mats, wo, wi_or_u, n, out);
    return cudaGetLastError();
}

cudaError_t launch_medium_tr_batch(const DevScene &S, int medium_id, const float *seg, const uint64_t *seeds,
                                   uint32_t n, float *out, cudaStream_t st)
{
    if(n == 0)
        return cudaSuccess;
    k_medium_tr_batch<<<(n + 127) / 128, 128, 0, st>>>(S, medium_id, seg, seeds, n, out);
    return cudaGetLastError();
}

} // namespace bt
