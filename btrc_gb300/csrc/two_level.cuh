// Two-level traversal: a top-level 8-wide tree over instance boxes and one object-space
// tree per geometry, the form of the reference's OptiX IAS over per-geometry GASes
// (core/btrc/core/scene.cpp:196-209, common/btrc/utils/optix/context.cpp:106-148).
//
// The top level is an ordinary compressed tree whose leaf records are instance boxes
// (v0 = box low corner with the instance index in v0.w, v1 = box high corner). At a leaf
// the ray is taken into the instance's object space with its world-to-local matrix,
// every multiply and add explicitly rounded in the order of the host's Transform::point
// (((m0 x + m1 y) + m2 z) + m3), so the oracle reproduces the object-space ray bit for
// bit; the geometry's tree is then walked with that ray and the closest hit so far.
// Hits keep the (t, instance, primitive) order of the single-level form, so the result
// does not depend on the order instances are visited in. The stage and ray-batch kernels
// run this form inside the warp-refill traversal (traverse_refill with TWO); the
// per-thread walk below serves the per-path kernels (radiance-cache training paths).
#pragma once

#include <cstddef>

#include "device.h"
#include "traverse.cuh"

namespace bt {

// the object-space ray of instance matrix m (3 x 4, row-major)
__device__ __forceinline__ void object_ray(const float *m, const float o[3], const float d[3], float oo[3],
                                           float od[3])
{
#pragma unroll
    for(int r = 0; r < 3; ++r)
    {
        const float *row = m + r * 4;
        float v = __fmul_rn(row[0], o[0]);
        v = __fadd_rn(v, __fmul_rn(row[1], o[1]));
        v = __fadd_rn(v, __fmul_rn(row[2], o[2]));
        oo[r] = __fadd_rn(v, row[3]);
        float w = __fmul_rn(row[0], d[0]);
        w = __fadd_rn(w, __fmul_rn(row[1], d[1]));
        od[r] = __fadd_rn(w, __fmul_rn(row[2], d[2]));
    }
}

// Walks one geometry's tree from `root` with an object-space ray; candidates carry the
// instance index. Returns true on the first hit when ANY.
template<bool ANY>
__device__ __forceinline__ bool walk_geometry(const TravRay &r, uint32_t root, uint32_t inst, const DevScene &S,
                                              ClosestResult &best, uint32_t *err)
{
    const float4 *nodes4 = reinterpret_cast<const float4 *>(S.blas_nodes);
    const float4 *tris4 = reinterpret_cast<const float4 *>(S.blas_tris);
    uint2 stack[STACK_SIZE];
    int sp = 0;
    uint2 ngroup = make_uint2(root, 0x80000000u);
    uint2 tgroup = make_uint2(0u, 0u);
    for(;;)
    {
        if(ngroup.y > 0x00ffffffu)
        {
            const int bit = 31 - __clz(ngroup.y);
            const uint32_t slot = (static_cast<uint32_t>(bit) - 24u) ^ r.oct_inv;
            const uint32_t rel = __popc(ngroup.y & ~(0xffffffffu << slot));
            const uint32_t ni = ngroup.x + rel;
            ngroup.y &= ~(1u << bit);
            if(ni >= S.blas_node_count)
            {
                atomicOr(err, 2u);
                return false;
            }
            if(ngroup.y > 0x00ffffffu)
            {
                if(sp >= STACK_SIZE)
                {
                    atomicOr(err, 1u);
                    return false;
                }
                stack[sp++] = ngroup;
            }
            uint32_t cbase, tbase, imask;
            const uint32_t hm = intersect_children(r, nodes4, ni, best.t, cbase, tbase, imask);
            ngroup = make_uint2(cbase, (hm & 0xff000000u) | imask);
            tgroup = make_uint2(tbase, hm & 0x00ffffffu);
        }
        while(tgroup.y != 0u)
        {
            const int tb = 31 - __clz(tgroup.y);
            tgroup.y &= ~(1u << tb);
            const uint32_t ti = tgroup.x + static_cast<uint32_t>(tb);
            if(ti >= S.blas_tri_count)
            {
                atomicOr(err, 2u);
                return false;
            }
            const float4 a = __ldg(tris4 + ti * 3 + 0);
            const float4 b = __ldg(tris4 + ti * 3 + 1);
            const float4 c = __ldg(tris4 + ti * 3 + 2);
            TriHit h;
            if(watertight(r, a, b, c, best.t, h))
            {
                const uint32_t prim = __float_as_uint(b.w);
                if(ANY)
                {
                    best.hit = true;
                    return true;
                }
                if(!best.hit || closer(h.t, inst, prim, best.t, best.inst, best.prim))
                {
                    best.hit = true;
                    best.t = h.t;
                    best.b1 = h.b1;
                    best.b2 = h.b2;
                    best.inst = inst;
                    best.prim = prim;
                }
            }
        }
        if(ngroup.y <= 0x00ffffffu)
        {
            if(sp == 0)
                return false;
            ngroup = stack[--sp];
        }
    }
}

// Closest (or, with ANY, any) hit in (0, t1] through the two-level form.
template<bool ANY>
__device__ __forceinline__ ClosestResult trace_two_level(const DevScene &S, const float o[3], const float d[3],
                                                         float t1, uint32_t *err)
{
    ClosestResult best;
    best.hit = false;
    best.t = t1;
    best.b1 = best.b2 = 0.0f;
    best.inst = best.prim = 0xffffffffu;
    if(S.node_count == 0)
        return best;
    const TravRay rw = make_trav_ray(o[0], o[1], o[2], d[0], d[1], d[2]);
    const float4 *nodes4 = reinterpret_cast<const float4 *>(S.nodes);
    const float4 *tris4 = reinterpret_cast<const float4 *>(S.tris);
    uint2 stack[STACK_SIZE];
    int sp = 0;
    uint2 ngroup = make_uint2(0u, 0x80000000u);
    uint2 tgroup = make_uint2(0u, 0u);
    for(;;)
    {
        if(ngroup.y > 0x00ffffffu)
        {
            const int bit = 31 - __clz(ngroup.y);
            const uint32_t slot = (static_cast<uint32_t>(bit) - 24u) ^ rw.oct_inv;
            const uint32_t rel = __popc(ngroup.y & ~(0xffffffffu << slot));
            const uint32_t ni = ngroup.x + rel;
            ngroup.y &= ~(1u << bit);
            if(ni >= S.node_count)
            {
                atomicOr(err, 2u);
                break;
            }
            if(ngroup.y > 0x00ffffffu)
            {
                if(sp >= STACK_SIZE)
                {
                    atomicOr(err, 1u);
                    break;
                }
                stack[sp++] = ngroup;
            }
            uint32_t cbase, tbase, imask;
            const uint32_t hm = intersect_children(rw, nodes4, ni, best.t, cbase, tbase, imask);
            ngroup = make_uint2(cbase, (hm & 0xff000000u) | imask);
            tgroup = make_uint2(tbase, hm & 0x00ffffffu);
        }
        while(tgroup.y != 0u)
        {
            const int tb = 31 - __clz(tgroup.y);
            tgroup.y &= ~(1u << tb);
            const uint32_t ti = tgroup.x + static_cast<uint32_t>(tb);
            if(ti >= S.tri_count)
            {
                atomicOr(err, 2u);
                tgroup.y = 0u;
                break;
            }
            const float4 blo = __ldg(tris4 + ti * 3), bhi = __ldg(tris4 + ti * 3 + 1);
            const uint32_t inst = __float_as_uint(blo.w);
            if(inst >= S.instance_count)
            {
                atomicOr(err, 2u);
                continue;
            }
            if(!box_hit(rw, blo, bhi, best.t))
                continue;
            const Instance &I = S.instances[inst];
            const uint32_t root = S.blas_root[I.geometry];
            if(root == 0xffffffffu)
                continue;
            float oo[3], od[3];
            object_ray(I.w2l, o, d, oo, od);
            const TravRay ro = make_trav_ray(oo[0], oo[1], oo[2], od[0], od[1], od[2]);
            if(walk_geometry<ANY>(ro, root, inst, S, best, err) && ANY)
                return best;
        }
        if(ngroup.y <= 0x00ffffffu)
        {
            if(sp == 0)
                break;
            ngroup = stack[--sp];
        }
    }
    return best;
}

// the two-level arrays for traverse_refill<..., TWO = true>
__host__ __device__ inline TwoLevelView two_level_view(const DevScene &S)
{
    TwoLevelView v;
    v.blas_nodes4 = reinterpret_cast<const float4 *>(S.blas_nodes);
    v.blas_tris4 = reinterpret_cast<const float4 *>(S.blas_tris);
    v.blas_root = S.blas_root;
    v.inst_rec = reinterpret_cast<const float *>(S.instances);
    v.inst_stride = static_cast<uint32_t>(sizeof(Instance) / sizeof(float));
    v.inst_geometry = static_cast<uint32_t>(offsetof(Instance, geometry) / sizeof(float));
    v.inst_count = S.instance_count;
    return v;
}

// per-thread closest / any hit for either form of the scene's acceleration structure
__device__ __forceinline__ ClosestResult scene_closest(const DevScene &S, const float o[3], const float d[3],
                                                       float t1, uint32_t *err)
{
    if(S.two_level)
        return trace_two_level<false>(S, o, d, t1, err);
    return trace_closest(make_trav_ray(o[0], o[1], o[2], d[0], d[1], d[2]), t1,
                         reinterpret_cast<const float4 *>(S.nodes), reinterpret_cast<const float4 *>(S.tris),
                         S.node_count, err);
}

__device__ __forceinline__ bool scene_any(const DevScene &S, const float o[3], const float d[3], float t1,
                                          uint32_t *err)
{
    if(S.two_level)
        return trace_two_level<true>(S, o, d, t1, err).hit;
    return trace_any(make_trav_ray(o[0], o[1], o[2], d[0], d[1], d[2]), t1, reinterpret_cast<const float4 *>(S.nodes),
                     reinterpret_cast<const float4 *>(S.tris), S.node_count, err);
}

} // namespace bt
