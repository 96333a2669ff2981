// 8-wide compressed-BVH traversal for sm_103a (closest hit and any hit).
//
// Node groups: a traversal entry is (base index, bit mask). Bits 24..31 mark child
// nodes still to visit (their slot XOR the ray octant, so the highest set bit is
// roughly the nearest child), bits 0..23 mark triangles of the current node. One
// group is pushed per tree level at most, so the per-thread stack needs no more
// entries than the tree has levels (the builder guarantees <= TRAVERSAL_STACK_SIZE).
//
// Triangle test: watertight ray/triangle intersection (Woop, Benthin, Wald, JCGT 2013)
// in FP32 with every multiply/add written as an explicitly rounded intrinsic, so the
// CPU oracle (compiled without FP contraction) reproduces t and the barycentrics bit
// for bit. Candidate order is a strict total order on (t, instance, primitive), which
// makes the closest hit independent of traversal order. Box tests are conservative:
// quantised boxes round outwards and the far distances (and the current closest t) are
// widened by 2^-20 relative.
#pragma once

#include <cstdint>

#include "bmath.h"
#include "layout.h"

namespace bt {

constexpr int STACK_SIZE = 32;
constexpr float BOX_EPS = 1.0f + 1.0f / 1048576.0f;

struct TravRay
{
    float ox, oy, oz;
    float dx, dy, dz;
    float idx, idy, idz;   // reciprocal direction, zero components replaced by +-1e-20
    uint32_t oct_inv;      // 7 - octant, octant bit k set when d[k] < 0
    int kx, ky, kz;        // watertight axis permutation
    float Sx, Sy, Sz;      // watertight shear
};

__device__ __forceinline__ float pick3(float x, float y, float z, int k)
{
    return k == 0 ? x : (k == 1 ? y : z);
}

__device__ __forceinline__ TravRay make_trav_ray(float ox, float oy, float oz, float dx, float dy, float dz)
{
    TravRay r;
    r.ox = ox; r.oy = oy; r.oz = oz;
    r.dx = dx; r.dy = dy; r.dz = dz;
    const float tiny = 1e-20f;
    const float sx = fabsf(dx) < tiny ? copysignf(tiny, dx) : dx;
    const float sy = fabsf(dy) < tiny ? copysignf(tiny, dy) : dy;
    const float sz = fabsf(dz) < tiny ? copysignf(tiny, dz) : dz;
    r.idx = __frcp_rn(sx);
    r.idy = __frcp_rn(sy);
    r.idz = __frcp_rn(sz);
    const uint32_t octant = (dx < 0.0f ? 1u : 0u) | (dy < 0.0f ? 2u : 0u) | (dz < 0.0f ? 4u : 0u);
    r.oct_inv = 7u - octant;

    const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    int kz = (ax >= ay) ? ((ax >= az) ? 0 : 2) : ((ay >= az) ? 1 : 2);
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    const float dkz = pick3(dx, dy, dz, kz);
    if(dkz < 0.0f)
    {
        const int t = kx;
        kx = ky;
        ky = t;
    }
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = __fdiv_rn(pick3(dx, dy, dz, kx), dkz);
    r.Sy = __fdiv_rn(pick3(dx, dy, dz, ky), dkz);
    r.Sz = __frcp_rn(dkz);
    return r;
}

struct TriHit
{
    float t, b1, b2;
};

// Returns true and fills h when the ray crosses the triangle at 0 < t <= tmax.
__device__ __forceinline__ bool watertight(const TravRay &r, float4 a, float4 b, float4 c, float tmax, TriHit &h)
{
    const float Axw = __fsub_rn(a.x, r.ox), Ayw = __fsub_rn(a.y, r.oy), Azw = __fsub_rn(a.z, r.oz);
    const float Bxw = __fsub_rn(b.x, r.ox), Byw = __fsub_rn(b.y, r.oy), Bzw = __fsub_rn(b.z, r.oz);
    const float Cxw = __fsub_rn(c.x, r.ox), Cyw = __fsub_rn(c.y, r.oy), Czw = __fsub_rn(c.z, r.oz);
    const float Akx = pick3(Axw, Ayw, Azw, r.kx), Aky = pick3(Axw, Ayw, Azw, r.ky), Akz = pick3(Axw, Ayw, Azw, r.kz);
    const float Bkx = pick3(Bxw, Byw, Bzw, r.kx), Bky = pick3(Bxw, Byw, Bzw, r.ky), Bkz = pick3(Bxw, Byw, Bzw, r.kz);
    const float Ckx = pick3(Cxw, Cyw, Czw, r.kx), Cky = pick3(Cxw, Cyw, Czw, r.ky), Ckz = pick3(Cxw, Cyw, Czw, r.kz);

    const float Ax = __fsub_rn(Akx, __fmul_rn(r.Sx, Akz));
    const float Ay = __fsub_rn(Aky, __fmul_rn(r.Sy, Akz));
    const float Bx = __fsub_rn(Bkx, __fmul_rn(r.Sx, Bkz));
    const float By = __fsub_rn(Bky, __fmul_rn(r.Sy, Bkz));
    const float Cx = __fsub_rn(Ckx, __fmul_rn(r.Sx, Ckz));
    const float Cy = __fsub_rn(Cky, __fmul_rn(r.Sy, Ckz));

    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if(U == 0.0f || V == 0.0f || W == 0.0f)
    {
        // exact products of floats in FP64, one rounding for the difference
        U = __double2float_rn(__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx)));
        V = __double2float_rn(__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx)));
        W = __double2float_rn(__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax)));
    }
    if((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f))
        return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if(det == 0.0f)
        return false;
    const float Az = __fmul_rn(r.Sz, Akz);
    const float Bz = __fmul_rn(r.Sz, Bkz);
    const float Cz = __fmul_rn(r.Sz, Ckz);
    const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    const float rcp = __frcp_rn(det);
    const float t = __fmul_rn(T, rcp);
    if(!(t > 0.0f && t <= tmax))
        return false;
    h.t = t;
    h.b1 = __fmul_rn(V, rcp);
    h.b2 = __fmul_rn(W, rcp);
    return true;
}

// Three-input FP32 min / max (sm_100 and later): one instruction instead of two.
__device__ __forceinline__ float max3f(float a, float b, float c)
{
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

__device__ __forceinline__ float min3f(float a, float b, float c)
{
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// 1 + b 2^-15 for byte j of w: the byte in mantissa bits 8..15 of 1.0f (0x3F80bb00), one
// byte permute and no arithmetic
__device__ __forceinline__ float byte_mant(uint32_t w, int j)
{
    return __uint_as_float(__byte_perm(w, 0x3F800000u, 0x7604u + (static_cast<uint32_t>(j) << 4)));
}

// Intersects the 8 children of a node. Returns the hit mask: bits 24..31 child nodes
// (slot ^ oct_inv), bits 0..23 triangles relative to tri_base.
__device__ __forceinline__ uint32_t intersect_children(const TravRay &r, const float4 *__restrict__ nodes4,
                                                      uint32_t ni, float tcur, uint32_t &child_base,
                                                      uint32_t &tri_base, uint32_t &imask)
{
    const float4 n0 = __ldg(nodes4 + ni * 5 + 0);
    const uint4 n1 = __ldg(reinterpret_cast<const uint4 *>(nodes4) + ni * 5 + 1);
    const uint4 n2 = __ldg(reinterpret_cast<const uint4 *>(nodes4) + ni * 5 + 2);
    const uint4 n3 = __ldg(reinterpret_cast<const uint4 *>(nodes4) + ni * 5 + 3);
    const uint4 n4 = __ldg(reinterpret_cast<const uint4 *>(nodes4) + ni * 5 + 4);
    const uint32_t ew = __float_as_uint(n0.w);
    imask = ew >> 24;
    child_base = n1.x;
    tri_base = n1.y;
    // Child plane k of an axis lies at n0 + k 2^e (k a byte, 2^e the node's grid step).
    // With F_k = 1 + k 2^-15 (the byte placed in mantissa bits 8..15 of 1.0f: one byte
    // permute), its distance along the ray is fma(F_k, A, C), A = 2^15 2^e / d exact and
    // C = (n0 - o) / d - A, since F_k A = A + k 2^e / d exactly inside the fma. C carries
    // rounding errors of up to 2^-23 (|org| + |A|); near planes use C lowered and far
    // planes C raised by pad = 2^-20 (|org| + |A|), and far distances are widened by
    // BOX_EPS as before, so every child box stays conservative.
    const float adjx = __uint_as_float((ew & 0xffu) << 23) * r.idx;
    const float adjy = __uint_as_float(((ew >> 8) & 0xffu) << 23) * r.idy;
    const float adjz = __uint_as_float(((ew >> 16) & 0xffu) << 23) * r.idz;
    const float orgx = (n0.x - r.ox) * r.idx;
    const float orgy = (n0.y - r.oy) * r.idy;
    const float orgz = (n0.z - r.oz) * r.idz;
    const float Ax = adjx * 32768.0f, Ay = adjy * 32768.0f, Az = adjz * 32768.0f;
    const float Cx = orgx - Ax, Cy = orgy - Ay, Cz = orgz - Az;
    const float PAD = 1.0f / 1048576.0f;
    const float padx = (fabsf(orgx) + fabsf(Ax)) * PAD;
    const float pady = (fabsf(orgy) + fabsf(Ay)) * PAD;
    const float padz = (fabsf(orgz) + fabsf(Az)) * PAD;
    const float ncx = Cx - padx, ncy = Cy - pady, ncz = Cz - padz;
    // far planes use coefficients pre-scaled by BOX_EPS, so every far distance comes out
    // widened by 2^-20 relative without a multiply per child
    const float fAx = Ax * BOX_EPS, fAy = Ay * BOX_EPS, fAz = Az * BOX_EPS;
    const float fcx = fmaf(Cx, BOX_EPS, padx), fcy = fmaf(Cy, BOX_EPS, pady), fcz = fmaf(Cz, BOX_EPS, padz);
    const float tcur_e = tcur * BOX_EPS;
    const bool nx = r.idx < 0.0f, ny = r.idy < 0.0f, nz = r.idz < 0.0f;
    const uint32_t oct4 = r.oct_inv * 0x01010101u;

    uint32_t hitmask = 0;
#pragma unroll
    for(int half = 0; half < 2; ++half)
    {
        // four meta bytes decoded at once: inner children (bits 3 and 4 set) get their
        // slot XOR the ray octant as bit index, leaves their triangle offset; an empty
        // slot (meta 0) contributes no bits, so it needs no test of its own
        const uint32_t meta4 = half ? n1.w : n1.z;
        const uint32_t inner4 = (meta4 & (meta4 << 1)) & 0x10101010u;
        const uint32_t bitidx4 = (meta4 ^ (oct4 & ((inner4 >> 4) * 7u))) & 0x1f1f1f1fu;
        const uint32_t cbits4 = (meta4 >> 5) & 0x07070707u;
        const uint32_t qlox = half ? n2.y : n2.x, qloy = half ? n2.w : n2.z, qloz = half ? n3.y : n3.x;
        const uint32_t qhix = half ? n3.w : n3.z, qhiy = half ? n4.y : n4.x, qhiz = half ? n4.w : n4.z;
        const uint32_t xn = nx ? qhix : qlox, xf = nx ? qlox : qhix;
        const uint32_t yn = ny ? qhiy : qloy, yf = ny ? qloy : qhiy;
        const uint32_t zn = nz ? qhiz : qloz, zf = nz ? qloz : qhiz;
#pragma unroll
        for(int j = 0; j < 4; ++j)
        {
            const float tnx = fmaf(byte_mant(xn, j), Ax, ncx);
            const float tny = fmaf(byte_mant(yn, j), Ay, ncy);
            const float tnz = fmaf(byte_mant(zn, j), Az, ncz);
            const float tfx = fmaf(byte_mant(xf, j), fAx, fcx);
            const float tfy = fmaf(byte_mant(yf, j), fAy, fcy);
            const float tfz = fmaf(byte_mant(zf, j), fAz, fcz);
            const float tmin = fmaxf(max3f(tnx, tny, tnz), 0.0f);
            const float tmax = fminf(min3f(tfx, tfy, tfz), tcur_e);
            if(tmin <= tmax)
                hitmask |= __byte_perm(cbits4, 0u, 0x4440u + j) << __byte_perm(bitidx4, 0u, 0x4440u + j);
        }
    }
    return hitmask;
}

// Ray against an axis-aligned box [lo, hi] over (0, tmax], the interval widened by 2^-20
// relative on both ends (the distances carry rounding errors of ~2^-23 relative), so the
// test stays conservative at any distance from the ray origin, like the node test
__device__ __forceinline__ bool box_hit(const TravRay &r, const float4 &lo, const float4 &hi, float tmax)
{
    const float x0 = (lo.x - r.ox) * r.idx, x1 = (hi.x - r.ox) * r.idx;
    const float y0 = (lo.y - r.oy) * r.idy, y1 = (hi.y - r.oy) * r.idy;
    const float z0 = (lo.z - r.oz) * r.idz, z1 = (hi.z - r.oz) * r.idz;
    const float tn = fmaxf(max3f(fminf(x0, x1), fminf(y0, y1), fminf(z0, z1)) * (2.0f - BOX_EPS), 0.0f);
    const float tf = fminf(min3f(fmaxf(x0, x1), fmaxf(y0, y1), fmaxf(z0, z1)), tmax) * BOX_EPS;
    return tn <= tf;
}

// Lexicographic (t, inst, prim) comparison used for closest-hit ties.
__device__ __forceinline__ bool closer(float t, uint32_t inst, uint32_t prim, float bt, uint32_t binst, uint32_t bprim)
{
    if(t != bt)
        return t < bt;
    if(inst != binst)
        return inst < binst;
    return prim < bprim;
}

struct ClosestResult
{
    float t, b1, b2;
    uint32_t inst, prim;
    bool hit;
};

// Closest hit in (0, t1]. err is set when the stack would overflow (never for trees
// accepted by the builder).
__device__ __forceinline__ ClosestResult trace_closest(const TravRay &r, float t1, const float4 *__restrict__ nodes4,
                                                       const float4 *__restrict__ tris4, uint32_t node_count,
                                                       uint32_t *err, uint32_t *stats_nodes = nullptr,
                                                       uint32_t *stats_tris = nullptr)
{
    ClosestResult best;
    best.hit = false;
    best.t = t1;
    best.b1 = best.b2 = 0.0f;
    best.inst = best.prim = 0xffffffffu;
    if(node_count == 0)
        return best;

    uint2 stack[STACK_SIZE];
    int sp = 0;
    uint2 ngroup = make_uint2(0u, 0x80000000u);
    uint2 tgroup = make_uint2(0u, 0u);
    uint32_t n_nodes = 0, n_tris = 0;
    for(;;)
    {
        if(ngroup.y > 0x00ffffffu)
        {
            const int bit = 31 - __clz(ngroup.y);
            const uint32_t slot = (static_cast<uint32_t>(bit) - 24u) ^ r.oct_inv;
            const uint32_t rel = __popc(ngroup.y & ~(0xffffffffu << slot));
            const uint32_t ni = ngroup.x + rel;
            ngroup.y &= ~(1u << bit);
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
            const uint32_t hm = intersect_children(r, nodes4, ni, best.t, cbase, tbase, imask);
            ++n_nodes;
            ngroup = make_uint2(cbase, (hm & 0xff000000u) | imask);
            tgroup = make_uint2(tbase, hm & 0x00ffffffu);
        }
        while(tgroup.y != 0u)
        {
            const int tb = 31 - __clz(tgroup.y);
            tgroup.y &= ~(1u << tb);
            const uint32_t ti = tgroup.x + static_cast<uint32_t>(tb);
            const float4 a = __ldg(tris4 + ti * 3 + 0);
            const float4 b = __ldg(tris4 + ti * 3 + 1);
            const float4 c = __ldg(tris4 + ti * 3 + 2);
            ++n_tris;
            TriHit h;
            if(watertight(r, a, b, c, best.t, h))
            {
                const uint32_t inst = __float_as_uint(a.w), prim = __float_as_uint(b.w);
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
                break;
            ngroup = stack[--sp];
        }
    }
    if(stats_nodes)
    {
        *stats_nodes = n_nodes;
        *stats_tris = n_tris;
    }
    return best;
}

// Any hit in (0, t1].
__device__ __forceinline__ bool trace_any(const TravRay &r, float t1, const float4 *__restrict__ nodes4,
                                          const float4 *__restrict__ tris4, uint32_t node_count, uint32_t *err)
{
    if(node_count == 0)
        return false;
    uint2 stack[STACK_SIZE];
    int sp = 0;
    uint2 ngroup = make_uint2(0u, 0x80000000u);
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
            const uint32_t hm = intersect_children(r, nodes4, ni, t1, cbase, tbase, imask);
            ngroup = make_uint2(cbase, (hm & 0xff000000u) | imask);
            tgroup = make_uint2(tbase, hm & 0x00ffffffu);
        }
        while(tgroup.y != 0u)
        {
            const int tb = 31 - __clz(tgroup.y);
            tgroup.y &= ~(1u << tb);
            const uint32_t ti = tgroup.x + static_cast<uint32_t>(tb);
            const float4 a = __ldg(tris4 + ti * 3 + 0);
            const float4 b = __ldg(tris4 + ti * 3 + 1);
            const float4 c = __ldg(tris4 + ti * 3 + 2);
            TriHit h;
            if(watertight(r, a, b, c, t1, h))
                return true;
        }
        if(ngroup.y <= 0x00ffffffu)
        {
            if(sp == 0)
                break;
            ngroup = stack[--sp];
        }
    }
    return false;
}

} // namespace bt

namespace bt {

// Persistent traversal with warp-level ray refill. Every lane runs the same loop; a lane
// whose ray has finished becomes idle, and once at least `refill` lanes of the warp are
// idle (or no lane is busy) the idle lanes take the next rays from a global cursor with
// one atomic per warp. Each loop iteration advances every busy lane by one node, so
// lanes never wait for the slowest ray of their warp.
//
// Triangle tests are pooled across the warp: a lane's pending triangles (the leaf bits of
// its last node) wait until the warp has min_round of them, or until no busy lane could
// go on without its results; then up to 32 are queued in shared memory and each lane of
// the warp tests one queued (ray, triangle) pair with the owning lane's ray, read from
// shared memory. The owners merge their results by shuffles. A lane with pending
// triangles takes no node step. Testing a leaf's triangles one after the
// other, lane by lane, ran with ~3 of 32 lanes active; pooled, a round runs with as
// many lanes as the warp has tests. Results are those of sequential testing: the
// closest hit is a strict total order on (t, instance, primitive).
//
// The kernel launches 128-thread blocks (TRAVERSE_WARPS warps, one shared-memory slice
// each), and all 32 lanes of a warp enter (the warp-wide votes use the full mask).
//   fetch(i, o, d, t1, root): load ray i;  emit(i, hit): store its result
constexpr int REFILL_LANES = 8;  // idle lanes that trigger a warp refill (measured best of 4/8/12/16/24)
constexpr int TRAVERSE_BLOCK = 128;
constexpr int TRAVERSE_WARPS = TRAVERSE_BLOCK / 32;
// queue entry: owner lane in bits 27..31, triangle record index in bits 0..26
constexpr uint32_t TRI_INDEX_BITS = 27;
constexpr uint32_t MAX_POOLED_TRIANGLES = 1u << TRI_INDEX_BITS;

// The two-level form (TWO): nodes4 / tris4 are the top level, whose leaf records are
// instance boxes (instance index in v0.w). A lane with pending instance leaves enters one
// at a time: it pushes its top-level node group and a marker entry (base | 2^31: node
// indices never set that bit) holding the remaining instances, takes its ray into the
// instance's object space (multiplies and adds rounded in the host transform's order),
// and walks the geometry's tree from its root; pooled triangle tests then use the
// object-space ray from shared memory like any other, and the owner stamps its
// instance on the results. Popping the marker restores the world ray.
struct TwoLevelView
{
    const float4 *blas_nodes4;
    const float4 *blas_tris4;
    const uint32_t *blas_root;
    const float *inst_rec;     // Instance records viewed as floats (w2l at offset 12)
    uint32_t inst_stride;      // floats per Instance record
    uint32_t inst_geometry;    // float offset of Instance::geometry
    uint32_t inst_count;
};
constexpr uint32_t MARKER_BIT = 0x80000000u;

// fetch(i, o, d, t1, root) loads ray i; root (0 unless fetch sets it) is the node the
// ray starts from, so that one node array can hold several BVHs
template<bool ANY, bool COUNT = false, bool TWO = false, typename Fetch, typename Emit>
__device__ __forceinline__ void traverse_refill(const float4 *__restrict__ nodes4, const float4 *__restrict__ tris4,
                                                uint32_t node_count, uint32_t *cursor, uint32_t n, int refill,
                                                uint32_t *err, Fetch fetch, Emit emit,
                                                uint64_t *node_visits = nullptr, uint64_t *tri_tests = nullptr,
                                                int min_round = 1, const TwoLevelView tl = TwoLevelView{})
{
    // per lane: (ox, oy, oz, Sx), (Sy, Sz, kx | ky << 2 | kz << 4, tmax); per warp: the queue
    __shared__ float4 s_ray0[TRAVERSE_WARPS][32];
    __shared__ float4 s_ray1[TRAVERSE_WARPS][32];
    __shared__ uint32_t s_queue[TRAVERSE_WARPS][32];
    uint64_t visits = 0, tests = 0;
    const uint32_t FULL = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = threadIdx.x >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const float NO_HIT = __int_as_float(0x7f800000);
    int state = 0;  // 0 idle, 1 busy, 2 exhausted
    uint32_t ray = 0;
    TravRay r;
    ClosestResult best;
    constexpr int STACK = TWO ? 2 * STACK_SIZE : STACK_SIZE;
    uint2 stack[STACK];
    int sp = 0;
    uint2 ngroup = make_uint2(0u, 0u);
    uint2 tgroup = make_uint2(0u, 0u);
    // two-level state: world ray, whether the lane is inside an instance, which one
    float wo[3] = { 0.0f, 0.0f, 0.0f }, wd[3] = { 0.0f, 0.0f, 0.0f };
    bool inside = false;
    uint32_t cur_inst = 0;
    const float4 *const leaf_tris4 = TWO ? tl.blas_tris4 : tris4;
    for(;;)
    {
        const uint32_t idle = __ballot_sync(FULL, state == 0);
        const uint32_t busy = __ballot_sync(FULL, state == 1);
        if(idle != 0u && (__popc(idle) >= refill || busy == 0u))
        {
            const uint32_t leader = __ffs(idle) - 1u;
            uint32_t base = 0;
            if(lane == leader)
                base = atomicAdd(cursor, static_cast<uint32_t>(__popc(idle)));
            base = __shfl_sync(FULL, base, leader);
            if(state == 0)
            {
                const uint32_t mine = base + static_cast<uint32_t>(__popc(idle & lt_mask));
                if(mine < n)
                {
                    float o[3], d[3], t1;
                    uint32_t root = 0;
                    fetch(mine, o, d, t1, root);
                    r = make_trav_ray(o[0], o[1], o[2], d[0], d[1], d[2]);
                    if(TWO)
                    {
#pragma unroll
                        for(int k = 0; k < 3; ++k)
                        {
                            wo[k] = o[k];
                            wd[k] = d[k];
                        }
                        inside = false;
                    }
                    ray = mine;
                    best.hit = false;
                    best.t = t1;
                    best.b1 = best.b2 = 0.0f;
                    best.inst = best.prim = 0xffffffffu;
                    sp = 0;
                    ngroup = make_uint2(root, node_count ? 0x80000000u : 0u);
                    tgroup = make_uint2(0u, 0u);
                    state = 1;
                    s_ray0[warp][lane] = make_float4(r.ox, r.oy, r.oz, r.Sx);
                    s_ray1[warp][lane] =
                        make_float4(r.Sy, r.Sz, __int_as_float(r.kx | (r.ky << 2) | (r.kz << 4)), t1);
                }
                else
                    state = 2;
            }
        }
        if(__all_sync(FULL, state == 2))
            break;

        // two-level: a lane at the top level with pending instance leaves enters one
        if(TWO && state == 1 && !inside && tgroup.y != 0u)
        {
            const int tb = 31 - __clz(tgroup.y);
            tgroup.y &= ~(1u << tb);
            const uint32_t ti = tgroup.x + static_cast<uint32_t>(tb);
            const float4 blo = __ldg(tris4 + ti * 3), bhi = __ldg(tris4 + ti * 3 + 1);
            const uint32_t inst = __float_as_uint(blo.w);
            const float *rec = tl.inst_rec + static_cast<size_t>(min(inst, tl.inst_count - 1u)) * tl.inst_stride;
            uint32_t root = inst < tl.inst_count ? tl.blas_root[__float_as_int(rec[tl.inst_geometry])] : 0xffffffffu;
            if(inst >= tl.inst_count)
                atomicOr(err, 2u);
            // the instance's own box (a leaf slot's box covers up to three): the box is
            // widened at build time far beyond the rounding of this test
            if(root != 0xffffffffu && !box_hit(r, blo, bhi, best.t))
                root = 0xffffffffu;
            if(root != 0xffffffffu)
            {
                if(sp + 2 > STACK)
                {
                    atomicOr(err, 1u);
                    ngroup = make_uint2(0u, 0u);
                    tgroup = make_uint2(0u, 0u);
                    sp = 0;
                }
                else
                {
                    if(ngroup.y > 0x00ffffffu)
                        stack[sp++] = ngroup;
                    stack[sp++] = make_uint2(tgroup.x | MARKER_BIT, tgroup.y);
                    float oo[3], od[3];
#pragma unroll
                    for(int rr = 0; rr < 3; ++rr)
                    {
                        const float *row = rec + 12 + rr * 4;
                        float v = __fmul_rn(row[0], wo[0]);
                        v = __fadd_rn(v, __fmul_rn(row[1], wo[1]));
                        v = __fadd_rn(v, __fmul_rn(row[2], wo[2]));
                        oo[rr] = __fadd_rn(v, row[3]);
                        float w = __fmul_rn(row[0], wd[0]);
                        w = __fadd_rn(w, __fmul_rn(row[1], wd[1]));
                        od[rr] = __fadd_rn(w, __fmul_rn(row[2], wd[2]));
                    }
                    r = make_trav_ray(oo[0], oo[1], oo[2], od[0], od[1], od[2]);
                    s_ray0[warp][lane] = make_float4(r.ox, r.oy, r.oz, r.Sx);
                    s_ray1[warp][lane] =
                        make_float4(r.Sy, r.Sz, __int_as_float(r.kx | (r.ky << 2) | (r.kz << 4)), best.t);
                    inside = true;
                    cur_inst = inst;
                    ngroup = make_uint2(root, 0x80000000u);
                    tgroup = make_uint2(0u, 0u);
                }
            }
        }
        // node step: busy lanes without pending triangles
        else if(state == 1 && tgroup.y == 0u && ngroup.y > 0x00ffffffu)
        {
            if(COUNT)
                ++visits;
            const int bit = 31 - __clz(ngroup.y);
            const uint32_t slot = (static_cast<uint32_t>(bit) - 24u) ^ r.oct_inv;
            const uint32_t rel = __popc(ngroup.y & ~(0xffffffffu << slot));
            const uint32_t ni = ngroup.x + rel;
            ngroup.y &= ~(1u << bit);
            bool overflow = false;
            if(ngroup.y > 0x00ffffffu)
            {
                if(sp >= STACK)
                {
                    atomicOr(err, 1u);
                    overflow = true;
                }
                else
                    stack[sp++] = ngroup;
            }
            if(overflow)
            {
                ngroup = make_uint2(0u, 0u);
                tgroup = make_uint2(0u, 0u);
                sp = 0;
            }
            else
            {
                uint32_t cbase, tbase, imask;
                const uint32_t hm =
                    intersect_children(r, TWO && inside ? tl.blas_nodes4 : nodes4, ni, best.t, cbase, tbase, imask);
                ngroup = make_uint2(cbase, (hm & 0xff000000u) | imask);
                tgroup = make_uint2(tbase, hm & 0x00ffffffu);
            }
        }

        // triangle round (all lanes). A round runs once min_round tests are pending, or
        // when no busy lane could make progress without one (every busy lane waits on
        // its triangles); queue positions come from a warp prefix sum of the counts.
        // (two-level: only lanes inside an instance hold triangles; instance leaves are
        // entered, not tested)
        const bool pooling = !TWO || inside;
        const uint32_t cnt = pooling ? static_cast<uint32_t>(__popc(tgroup.y)) : 0u;
        const uint32_t total = __reduce_add_sync(FULL, cnt);
        bool found_any = false;
        const uint32_t steppers = __ballot_sync(FULL, state == 1 && (tgroup.y == 0u || !pooling));
        const bool round = total != 0u && (total >= static_cast<uint32_t>(min_round) || steppers == 0u);
        if(round)
        {
            uint32_t incl = cnt;
#pragma unroll
            for(int off = 1; off < 32; off <<= 1)
            {
                const uint32_t v = __shfl_up_sync(FULL, incl, off);
                if(lane >= static_cast<uint32_t>(off))
                    incl += v;
            }
            const uint32_t excl = incl - cnt;
            const uint32_t take = excl >= 32u ? 0u : min(cnt, 32u - excl);
            if(take != 0u)
            {
                uint32_t bits = tgroup.y;
                for(uint32_t k = 0; k < take; ++k)
                {
                    const int tb = 31 - __clz(bits);
                    bits &= ~(1u << tb);
                    s_queue[warp][excl + k] = (lane << TRI_INDEX_BITS) | (tgroup.x + static_cast<uint32_t>(tb));
                }
                tgroup.y = bits;
                s_ray1[warp][lane].w = best.t;
                if(COUNT)
                    tests += take;
            }
            __syncwarp();
            // tester: queue entry `lane`
            float ht = NO_HIT, hb1 = 0.0f, hb2 = 0.0f;
            uint32_t hinst = 0u, hprim = 0u;
            if(lane < min(total, 32u))
            {
                const uint32_t e = s_queue[warp][lane];
                const uint32_t owner = e >> TRI_INDEX_BITS, ti = e & (MAX_POOLED_TRIANGLES - 1u);
                const float4 q0 = s_ray0[warp][owner], q1 = s_ray1[warp][owner];
                TravRay tr;
                tr.ox = q0.x; tr.oy = q0.y; tr.oz = q0.z;
                tr.Sx = q0.w; tr.Sy = q1.x; tr.Sz = q1.y;
                const int kk = __float_as_int(q1.z);
                tr.kx = kk & 3; tr.ky = (kk >> 2) & 3; tr.kz = (kk >> 4) & 3;
                const float4 a = __ldg(leaf_tris4 + ti * 3 + 0);
                const float4 b = __ldg(leaf_tris4 + ti * 3 + 1);
                const float4 c = __ldg(leaf_tris4 + ti * 3 + 2);
                TriHit h;
                if(watertight(tr, a, b, c, q1.w, h))
                {
                    ht = h.t;
                    hb1 = h.b1;
                    hb2 = h.b2;
                    hinst = __float_as_uint(a.w);
                    hprim = __float_as_uint(b.w);
                }
            }
            // two-level: object-space records carry no instance; the owner's is the one
            const uint32_t my_inst = cur_inst;
            // owners merge their entries [excl, excl + take): the smallest t by shuffling
            // t alone, then the winner's record; equal t within one owner's entries (a ray
            // through a shared edge) takes the exact (t, instance, primitive) order
            const uint32_t rounds = __reduce_max_sync(FULL, take);
            if(ANY)
            {
                for(uint32_t k = 0; k < rounds; ++k)
                {
                    const float ct = __shfl_sync(FULL, ht, static_cast<int>(min(excl + k, 31u)));
                    if(k < take && ct != NO_HIT)
                        found_any = true;
                }
            }
            else
            {
                float mt = NO_HIT;
                uint32_t msrc = lane;
                bool tie = false;
                for(uint32_t k = 0; k < rounds; ++k)
                {
                    const uint32_t src = min(excl + k, 31u);
                    const float ct = __shfl_sync(FULL, ht, static_cast<int>(src));
                    if(k < take && ct != NO_HIT)
                    {
                        if(ct < mt)
                        {
                            mt = ct;
                            msrc = src;
                            tie = false;
                        }
                        else if(ct == mt)
                            tie = true;
                    }
                }
                if(__ballot_sync(FULL, tie) == 0u)
                {
                    const float cb1 = __shfl_sync(FULL, hb1, static_cast<int>(msrc));
                    const float cb2 = __shfl_sync(FULL, hb2, static_cast<int>(msrc));
                    const uint32_t ci = TWO ? my_inst : __shfl_sync(FULL, hinst, static_cast<int>(msrc));
                    const uint32_t cp = __shfl_sync(FULL, hprim, static_cast<int>(msrc));
                    if(mt != NO_HIT && (!best.hit || closer(mt, ci, cp, best.t, best.inst, best.prim)))
                    {
                        best.hit = true;
                        best.t = mt;
                        best.b1 = cb1;
                        best.b2 = cb2;
                        best.inst = ci;
                        best.prim = cp;
                    }
                }
                else
                {
                    for(uint32_t k = 0; k < rounds; ++k)
                    {
                        const int src = static_cast<int>(min(excl + k, 31u));
                        const float ct = __shfl_sync(FULL, ht, src);
                        const float cb1 = __shfl_sync(FULL, hb1, src);
                        const float cb2 = __shfl_sync(FULL, hb2, src);
                        const uint32_t ci = TWO ? my_inst : __shfl_sync(FULL, hinst, src);
                        const uint32_t cp = __shfl_sync(FULL, hprim, src);
                        if(k < take && ct != NO_HIT &&
                           (!best.hit || closer(ct, ci, cp, best.t, best.inst, best.prim)))
                        {
                            best.hit = true;
                            best.t = ct;
                            best.b1 = cb1;
                            best.b2 = cb2;
                            best.inst = ci;
                            best.prim = cp;
                        }
                    }
                }
            }
        }
        if(state != 1)
            continue;
        if(ANY && found_any)
        {
            best.hit = true;
            emit(ray, best);
            tgroup.y = 0u;
            state = 0;
            continue;
        }
        if(tgroup.y == 0u && ngroup.y <= 0x00ffffffu)
        {
            if(sp == 0)
            {
                emit(ray, best);
                state = 0;
            }
            else
            {
                const uint2 e = stack[--sp];
                if(TWO && (e.x & MARKER_BIT))
                {
                    // back at the top level: the world ray and the remaining instances
                    r = make_trav_ray(wo[0], wo[1], wo[2], wd[0], wd[1], wd[2]);
                    s_ray0[warp][lane] = make_float4(r.ox, r.oy, r.oz, r.Sx);
                    s_ray1[warp][lane] =
                        make_float4(r.Sy, r.Sz, __int_as_float(r.kx | (r.ky << 2) | (r.kz << 4)), best.t);
                    inside = false;
                    ngroup = make_uint2(0u, 0u);
                    tgroup = make_uint2(e.x & ~MARKER_BIT, e.y);
                }
                else
                    ngroup = e;
            }
        }
    }
    if(COUNT)
    {
        *node_visits += visits;
        *tri_tests += tests;
    }
}

} // namespace bt
