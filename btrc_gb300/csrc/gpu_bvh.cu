// Device BVH builder (see gpu_bvh.h): PLOC binary tree, bottom-up 8-wide collapse,
// level-by-level emission of 80-byte compressed nodes.
#include "gpu_bvh.h"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cmath>
#include <vector>

#include "bvh.h"

namespace bt {

namespace {

constexpr int BLOCK = 256;
// PLOC neighbour window on each side. On the 1080p terrain, radii 8, 16, 24, 32 and 48
// gave frames of 142.1, 143.5, 143.4, 144.7 and 144.7 ms (host binned SAH: 130.1 ms) at
// equal build times (16.5-18.8 ms), so the smallest window stays.
constexpr int RADIUS = 8;
constexpr uint32_t MAX_LEAF_TRIS = 3;   // one wide-node leaf slot
constexpr float COST_NODE = 1.0f;       // the host collapse's weights (bvh.cpp)
constexpr float COST_TRI = 0.4f;
constexpr int MAX_ITERATIONS = 1 << 15;

// binary node: two float4, (lo.xyz, left) and (hi.xyz, right); a leaf has left = -1 and
// right = its triangle's index in the input array
__device__ __forceinline__ int32_t f2i(float f) { return __float_as_int(f); }
__device__ __forceinline__ float i2f(int32_t i) { return __int_as_float(i); }

// order-preserving map of floats to unsigned integers, for atomic min / max
__device__ __forceinline__ uint32_t ord(float f)
{
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unord(uint32_t u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__device__ __forceinline__ void tri_box(const TriRec &t, float *lo, float *hi)
{
    lo[0] = fminf(fminf(t.v0x, t.v1x), t.v2x);
    lo[1] = fminf(fminf(t.v0y, t.v1y), t.v2y);
    lo[2] = fminf(fminf(t.v0z, t.v1z), t.v2z);
    hi[0] = fmaxf(fmaxf(t.v0x, t.v1x), t.v2x);
    hi[1] = fmaxf(fmaxf(t.v0y, t.v1y), t.v2y);
    hi[2] = fmaxf(fmaxf(t.v0z, t.v1z), t.v2z);
}

__global__ void __launch_bounds__(BLOCK) k_centroid_bounds(const TriRec *__restrict__ tris, uint32_t n,
                                                           uint32_t *__restrict__ cb)
{
    float lo[3] = { MAX_FLOAT, MAX_FLOAT, MAX_FLOAT }, hi[3] = { -MAX_FLOAT, -MAX_FLOAT, -MAX_FLOAT };
    for(uint32_t i = blockIdx.x * BLOCK + threadIdx.x; i < n; i += gridDim.x * BLOCK)
    {
        float a[3], b[3];
        tri_box(tris[i], a, b);
        for(int k = 0; k < 3; ++k)
        {
            const float c = 0.5f * (a[k] + b[k]);
            lo[k] = fminf(lo[k], c);
            hi[k] = fmaxf(hi[k], c);
        }
    }
    for(int off = 16; off > 0; off >>= 1)
        for(int k = 0; k < 3; ++k)
        {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], off));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], off));
        }
    if((threadIdx.x & 31) == 0)
        for(int k = 0; k < 3; ++k)
        {
            atomicMin(&cb[k], ord(lo[k]));
            atomicMax(&cb[3 + k], ord(hi[k]));
        }
}

// 21 bits of x spread to every third bit of a 64-bit word
__device__ __forceinline__ uint64_t spread3(uint32_t v)
{
    uint64_t x = v & 0x1fffffu;
    x = (x | x << 32) & 0x1f00000000ffffull;
    x = (x | x << 16) & 0x1f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

__global__ void __launch_bounds__(BLOCK) k_morton(const TriRec *__restrict__ tris, uint32_t n,
                                                  const uint32_t *__restrict__ cb, uint64_t *__restrict__ keys,
                                                  uint32_t *__restrict__ vals)
{
    const uint32_t i = blockIdx.x * BLOCK + threadIdx.x;
    if(i >= n)
        return;
    float a[3], b[3];
    tri_box(tris[i], a, b);
    uint32_t q[3];
    for(int k = 0; k < 3; ++k)
    {
        const float lo = unord(cb[k]), hi = unord(cb[3 + k]);
        const float ext = hi - lo;
        const float c = 0.5f * (a[k] + b[k]);
        const float s = ext > 0.0f ? (c - lo) / ext * 2097151.0f : 0.0f;
        q[k] = s > 0.0f ? static_cast<uint32_t>(fminf(s, 2097151.0f)) : 0u;
    }
    keys[i] = spread3(q[0]) | spread3(q[1]) << 1 | spread3(q[2]) << 2;
    vals[i] = i;
}

// leaves in Morton order become the first clusters
__global__ void __launch_bounds__(BLOCK) k_leaves(const TriRec *__restrict__ tris, const uint32_t *__restrict__ perm,
                                                  uint32_t n, float4 *__restrict__ nlo, float4 *__restrict__ nhi,
                                                  uint32_t *__restrict__ cid, float4 *__restrict__ clo,
                                                  float4 *__restrict__ chi)
{
    const uint32_t p = blockIdx.x * BLOCK + threadIdx.x;
    if(p >= n)
        return;
    const uint32_t t = perm[p];
    float a[3], b[3];
    tri_box(tris[t], a, b);
    nlo[p] = make_float4(a[0], a[1], a[2], i2f(-1));
    nhi[p] = make_float4(b[0], b[1], b[2], i2f(static_cast<int32_t>(t)));
    cid[p] = p;
    clo[p] = make_float4(a[0], a[1], a[2], 0.0f);
    chi[p] = make_float4(b[0], b[1], b[2], 0.0f);
}

__device__ __forceinline__ uint32_t pair_hash(uint32_t lo, uint32_t hi)
{
    uint32_t h = lo * 0x9e3779b1u ^ (hi + 0x7f4a7c15u) * 0x85ebca77u;
    h ^= h >> 15;
    h *= 0xc2b2ae3du;
    h ^= h >> 13;
    return h;
}

// nearest neighbour of every cluster within RADIUS positions: least surface area of the
// union. Ties go to the pair of least (hash, low index, high index), the same order seen
// from both ends of a pair, so the globally least pair is always mutual and every
// iteration merges at least one pair.
__global__ void __launch_bounds__(BLOCK) k_nearest(uint32_t m, const float4 *__restrict__ clo,
                                                   const float4 *__restrict__ chi, uint32_t *__restrict__ nn)
{
    __shared__ float slo[3][BLOCK + 2 * RADIUS];
    __shared__ float shi[3][BLOCK + 2 * RADIUS];
    const int base = blockIdx.x * BLOCK;
    for(int k = threadIdx.x; k < BLOCK + 2 * RADIUS; k += BLOCK)
    {
        const int g = base - RADIUS + k;
        float4 l = make_float4(0.0f, 0.0f, 0.0f, 0.0f), h = l;
        if(g >= 0 && g < static_cast<int>(m))
        {
            l = clo[g];
            h = chi[g];
        }
        slo[0][k] = l.x; slo[1][k] = l.y; slo[2][k] = l.z;
        shi[0][k] = h.x; shi[1][k] = h.y; shi[2][k] = h.z;
    }
    __syncthreads();
    const int i = base + threadIdx.x;
    if(i >= static_cast<int>(m))
        return;
    const int si = threadIdx.x + RADIUS;
    const float ax = slo[0][si], ay = slo[1][si], az = slo[2][si];
    const float bx = shi[0][si], by = shi[1][si], bz = shi[2][si];
    float best = __int_as_float(0x7f800000);
    uint32_t bh = 0xffffffffu, bl = 0xffffffffu, bu = 0xffffffffu;
    int bj = -1;
    for(int d = -RADIUS; d <= RADIUS; ++d)
    {
        const int j = i + d;
        if(d == 0 || j < 0 || j >= static_cast<int>(m))
            continue;
        const int sj = si + d;
        const float dx = __fsub_rn(fmaxf(bx, shi[0][sj]), fminf(ax, slo[0][sj]));
        const float dy = __fsub_rn(fmaxf(by, shi[1][sj]), fminf(ay, slo[1][sj]));
        const float dz = __fsub_rn(fmaxf(bz, shi[2][sj]), fminf(az, slo[2][sj]));
        const float area = __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx));
        const uint32_t lo = static_cast<uint32_t>(min(i, j)), hi = static_cast<uint32_t>(max(i, j));
        const uint32_t h = pair_hash(lo, hi);
        const bool better =
            area < best ||
            (area == best && (h < bh || (h == bh && (lo < bl || (lo == bl && hi < bu)))));
        if(better)
        {
            best = area;
            bh = h;
            bl = lo;
            bu = hi;
            bj = j;
        }
    }
    nn[i] = bj < 0 ? static_cast<uint32_t>(i) : static_cast<uint32_t>(bj);
}

// mutual nearest neighbours merge: the lower position takes the new node, the higher one
// leaves; keep[m] is cleared for the scan's total
__global__ void __launch_bounds__(BLOCK) k_merge(uint32_t m, uint32_t n, const uint32_t *__restrict__ nn,
                                                 uint32_t *__restrict__ cid, float4 *__restrict__ clo,
                                                 float4 *__restrict__ chi, float4 *__restrict__ nlo,
                                                 float4 *__restrict__ nhi, int32_t *__restrict__ parent,
                                                 uint32_t *__restrict__ counter, uint32_t *__restrict__ keep,
                                                 uint32_t *__restrict__ err)
{
    const uint32_t i = blockIdx.x * BLOCK + threadIdx.x;
    if(i == 0)
        keep[m] = 0;
    if(i >= m)
        return;
    const uint32_t j = nn[i];
    uint32_t k = 1;
    if(j != i && j < m && nn[j] == i)
    {
        if(i < j)
        {
            const uint32_t slot = atomicAdd(counter, 1u);
            if(slot >= n - 1)
                atomicOr(err, 1u);
            else
            {
                const uint32_t node = n + slot;
                const float4 al = clo[i], ah = chi[i], bl = clo[j], bh = chi[j];
                const float4 lo = make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.0f);
                const float4 hi = make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.0f);
                const uint32_t a = cid[i], b = cid[j];
                nlo[node] = make_float4(lo.x, lo.y, lo.z, i2f(static_cast<int32_t>(a)));
                nhi[node] = make_float4(hi.x, hi.y, hi.z, i2f(static_cast<int32_t>(b)));
                parent[a] = static_cast<int32_t>(node);
                parent[b] = static_cast<int32_t>(node);
                cid[i] = node;
                clo[i] = lo;
                chi[i] = hi;
            }
        }
        else
            k = 0;
    }
    keep[i] = k;
}

__global__ void __launch_bounds__(BLOCK) k_compact(uint32_t m, const uint32_t *__restrict__ keep,
                                                   const uint32_t *__restrict__ pos, const uint32_t *__restrict__ cid,
                                                   const float4 *__restrict__ clo, const float4 *__restrict__ chi,
                                                   uint32_t *__restrict__ cid2, float4 *__restrict__ clo2,
                                                   float4 *__restrict__ chi2)
{
    const uint32_t i = blockIdx.x * BLOCK + threadIdx.x;
    if(i >= m || !keep[i])
        return;
    const uint32_t p = pos[i];
    cid2[p] = cid[i];
    clo2[p] = clo[i];
    chi2[p] = chi[i];
}

// collapse tables: C(q, i) = cost[q * 8 + i - 1], the least SAH cost of q's subtree over
// at most i slots; split[q * 8 + i - 1] the left child's share (0: as for i - 1)
struct Tables
{
    float *cost;
    uint8_t *split;
    uint8_t *split8;
    uint8_t *as_leaf;
    uint32_t *ntri;
};

__device__ __forceinline__ float node_area(const float4 &lo, const float4 &hi)
{
    if(lo.x > hi.x)
        return 0.0f;
    const double dx = (double)hi.x - lo.x, dy = (double)hi.y - lo.y, dz = (double)hi.z - lo.z;
    return static_cast<float>(2.0 * (dx * dy + dy * dz + dz * dx));
}

// the host builder's collapse_costs (bvh.cpp) for one internal node
__device__ void collapse_node(uint32_t q, const float4 *nlo, const float4 *nhi, Tables T)
{
    const float4 lo = __ldcg(&nlo[q]), hi = __ldcg(&nhi[q]);
    const uint32_t l = static_cast<uint32_t>(f2i(lo.w)), r = static_cast<uint32_t>(f2i(hi.w));
    const float A = node_area(lo, hi);
    const float INF = __int_as_float(0x7f800000);
    float cl[8], cr[8];
    for(int k = 0; k < 8; ++k)
    {
        cl[k] = __ldcg(&T.cost[static_cast<size_t>(l) * 8 + k]);
        cr[k] = __ldcg(&T.cost[static_cast<size_t>(r) * 8 + k]);
    }
    const uint32_t nt = __ldcg(&T.ntri[l]) + __ldcg(&T.ntri[r]);
    T.ntri[q] = nt;
    float dist[9];
    uint8_t arg[9] = {};
    for(int j = 2; j <= 8; ++j)
    {
        dist[j] = INF;
        for(int k = 1; k < j; ++k)
        {
            const float v = __fadd_rn(cl[k - 1], cr[j - k - 1]);
            if(v < dist[j])
            {
                dist[j] = v;
                arg[j] = static_cast<uint8_t>(k);
            }
        }
    }
    T.split8[q] = arg[8];
    const float c_internal = __fadd_rn(__fmul_rn(A, COST_NODE), dist[8]);
    const float c_leaf = nt <= MAX_LEAF_TRIS ? __fmul_rn(__fmul_rn(A, COST_TRI), static_cast<float>(nt)) : INF;
    T.as_leaf[q] = c_leaf <= c_internal ? 1 : 0;
    float *c = &T.cost[static_cast<size_t>(q) * 8];
    uint8_t *sp = &T.split[static_cast<size_t>(q) * 8];
    float prev = fminf(c_leaf, c_internal);
    c[0] = prev;
    sp[0] = 0;
    for(int i = 2; i <= 8; ++i)
    {
        if(dist[i] < prev)
        {
            prev = dist[i];
            sp[i - 1] = arg[i];
        }
        else
            sp[i - 1] = 0;
        c[i - 1] = prev;
    }
}

// bottom-up: one thread per leaf climbs while it is the second child to arrive
__global__ void __launch_bounds__(BLOCK) k_collapse(uint32_t n, const float4 *__restrict__ nlo,
                                                    const float4 *__restrict__ nhi, const int32_t *__restrict__ parent,
                                                    uint32_t *__restrict__ visits, Tables T)
{
    const uint32_t p = blockIdx.x * BLOCK + threadIdx.x;
    if(p >= n)
        return;
    {
        const float A = node_area(nlo[p], nhi[p]);
        const float c = __fmul_rn(A, COST_TRI);
        for(int k = 0; k < 8; ++k)
        {
            T.cost[static_cast<size_t>(p) * 8 + k] = c;
            T.split[static_cast<size_t>(p) * 8 + k] = 0;
        }
        T.split8[p] = 0;
        T.as_leaf[p] = 1;
        T.ntri[p] = 1;
    }
    int32_t x = parent[p];
    for(uint32_t guard = 0; x >= 0 && guard < 2 * n; ++guard)
    {
        __threadfence();
        if(atomicAdd(&visits[static_cast<uint32_t>(x) - n], 1u) == 0)
            return;
        __threadfence();
        collapse_node(static_cast<uint32_t>(x), nlo, nhi, T);
        x = parent[x];
    }
}

// the children of one wide node: binary subtrees by slot
struct KidSet
{
    int32_t kid[8];
    int8_t in_slot[8];
    uint32_t n;
    uint32_t n_internal;
    uint32_t n_tris;
    uint32_t pad;
};

__global__ void __launch_bounds__(BLOCK) k_kids(const uint32_t *__restrict__ level, uint32_t count,
                                                const float4 *__restrict__ nlo, const float4 *__restrict__ nhi,
                                                Tables T, KidSet *__restrict__ kids, uint32_t *__restrict__ ni,
                                                uint32_t *__restrict__ nt, uint32_t *__restrict__ err)
{
    const uint32_t i = blockIdx.x * BLOCK + threadIdx.x;
    if(i == 0)
    {
        ni[count] = 0;
        nt[count] = 0;
    }
    if(i >= count)
        return;
    KidSet w;
    w.n = 0;
    w.n_internal = 0;
    w.n_tris = 0;
    w.pad = 0;
    const uint32_t m = level[i];
    const int32_t ml = f2i(nlo[m].w);
    if(ml < 0)
        w.kid[w.n++] = static_cast<int32_t>(m);
    else
    {
        // expand (node, slots) pairs, left subtree first, as the host collapse does
        uint32_t st_node[16];
        int st_slots[16];
        int sp = 0;
        const int k8 = T.split8[m];
        st_node[sp] = static_cast<uint32_t>(f2i(nhi[m].w));
        st_slots[sp++] = 8 - k8;
        st_node[sp] = static_cast<uint32_t>(ml);
        st_slots[sp++] = k8;
        while(sp > 0)
        {
            const uint32_t x = st_node[--sp];
            int s = st_slots[sp];
            while(s >= 2 && T.split[static_cast<size_t>(x) * 8 + s - 1] == 0)
                --s;
            if(s <= 1)
            {
                if(w.n >= 8)
                {
                    atomicOr(err, 2u);
                    break;
                }
                w.kid[w.n++] = static_cast<int32_t>(x);
                continue;
            }
            if(sp + 2 > 16)
            {
                atomicOr(err, 2u);
                break;
            }
            const int k = T.split[static_cast<size_t>(x) * 8 + s - 1];
            st_node[sp] = static_cast<uint32_t>(f2i(nhi[x].w));
            st_slots[sp++] = s - k;
            st_node[sp] = static_cast<uint32_t>(f2i(nlo[x].w));
            st_slots[sp++] = k;
        }
    }
    // slot s prefers children far along (s&1 ? +x : -x, s&2 ? +y : -y, s&4 ? +z : -z);
    // the traversal visits slot == ray octant first
    float blo[3] = { MAX_FLOAT, MAX_FLOAT, MAX_FLOAT }, bhi[3] = { -MAX_FLOAT, -MAX_FLOAT, -MAX_FLOAT };
    for(uint32_t k = 0; k < w.n; ++k)
    {
        const float4 l = nlo[w.kid[k]], h = nhi[w.kid[k]];
        blo[0] = fminf(blo[0], l.x); blo[1] = fminf(blo[1], l.y); blo[2] = fminf(blo[2], l.z);
        bhi[0] = fmaxf(bhi[0], h.x); bhi[1] = fmaxf(bhi[1], h.y); bhi[2] = fmaxf(bhi[2], h.z);
    }
    double pc[3];
    for(int a = 0; a < 3; ++a)
        pc[a] = 0.5 * ((double)blo[a] + bhi[a]);
    double cost[8][8];
    for(uint32_t k = 0; k < w.n; ++k)
    {
        const float4 l = nlo[w.kid[k]], h = nhi[w.kid[k]];
        const double cc[3] = { 0.5 * ((double)l.x + h.x) - pc[0], 0.5 * ((double)l.y + h.y) - pc[1],
                               0.5 * ((double)l.z + h.z) - pc[2] };
        for(int s = 0; s < 8; ++s)
            cost[k][s] = ((s & 1) ? cc[0] : -cc[0]) + ((s & 2) ? cc[1] : -cc[1]) + ((s & 4) ? cc[2] : -cc[2]);
    }
    for(int s = 0; s < 8; ++s)
        w.in_slot[s] = -1;
    uint32_t done = 0;
    for(uint32_t round = 0; round < w.n; ++round)
    {
        int bk = -1, bs = -1;
        double bc = -__longlong_as_double(0x7ff0000000000000ll);
        for(uint32_t k = 0; k < w.n; ++k)
        {
            if(done >> k & 1)
                continue;
            for(int s = 0; s < 8; ++s)
                if(w.in_slot[s] < 0 && cost[k][s] > bc)
                {
                    bc = cost[k][s];
                    bk = static_cast<int>(k);
                    bs = s;
                }
        }
        if(bk < 0)
        {
            atomicOr(err, 2u);
            break;
        }
        done |= 1u << bk;
        w.in_slot[bs] = static_cast<int8_t>(bk);
    }
    for(uint32_t k = 0; k < w.n; ++k)
    {
        const int32_t c = w.kid[k];
        if(T.as_leaf[c])
            w.n_tris += T.ntri[c];
        else
            ++w.n_internal;
    }
    kids[i] = w;
    ni[i] = w.n_internal;
    nt[i] = w.n_tris;
}

// Smallest e with 255 * 2^e >= extent, clamped so that 2^e is a normal float (the host
// builder's quant_exponent).
__device__ int quant_exponent(double extent)
{
    if(!(extent > 0))
        return -126;
    if(!(extent < 1e300))
        return 127;
    int e = static_cast<int>(ceil(log2(extent / 255.0)));
    e = max(-200, min(200, e));
    for(int g = 0; g < 8 && ldexp(255.0, e) < extent; ++g)
        ++e;
    for(int g = 0; g < 8 && e > -126 && ldexp(255.0, e - 1) >= extent; ++g)
        --e;
    return max(-126, min(127, e));
}

__global__ void __launch_bounds__(BLOCK) k_emit(const uint32_t *__restrict__ level, uint32_t count,
                                                const KidSet *__restrict__ kids, const uint32_t *__restrict__ cbase,
                                                const uint32_t *__restrict__ tbase, uint32_t level_base,
                                                uint32_t next_base, uint32_t tri_cursor, const float4 *__restrict__ nlo,
                                                const float4 *__restrict__ nhi, Tables T,
                                                const TriRec *__restrict__ tris, uint32_t n,
                                                CWNode *__restrict__ out_nodes, uint32_t node_cap,
                                                TriRec *__restrict__ out_tris, uint32_t *__restrict__ next_level,
                                                uint32_t *__restrict__ err)
{
    const uint32_t i = blockIdx.x * BLOCK + threadIdx.x;
    if(i >= count)
        return;
    const KidSet &w = kids[i];
    const uint32_t child_base = next_base + cbase[i];
    const uint32_t tri_base = tri_cursor + tbase[i];
    if(level_base + i >= node_cap || child_base + w.n_internal > node_cap || tri_base + w.n_tris > n)
    {
        atomicOr(err, 4u);
        return;
    }
    float blo[3] = { MAX_FLOAT, MAX_FLOAT, MAX_FLOAT }, bhi[3] = { -MAX_FLOAT, -MAX_FLOAT, -MAX_FLOAT };
    for(uint32_t k = 0; k < w.n; ++k)
    {
        const float4 l = nlo[w.kid[k]], h = nhi[w.kid[k]];
        blo[0] = fminf(blo[0], l.x); blo[1] = fminf(blo[1], l.y); blo[2] = fminf(blo[2], l.z);
        bhi[0] = fmaxf(bhi[0], h.x); bhi[1] = fmaxf(bhi[1], h.y); bhi[2] = fmaxf(bhi[2], h.z);
    }
    CWNode node;
    node.px = blo[0];
    node.py = blo[1];
    node.pz = blo[2];
    int ex[3];
    for(int a = 0; a < 3; ++a)
        ex[a] = quant_exponent((double)bhi[a] - (double)blo[a]);
    node.ex = static_cast<uint8_t>(ex[0] + 127);
    node.ey = static_cast<uint8_t>(ex[1] + 127);
    node.ez = static_cast<uint8_t>(ex[2] + 127);
    node.imask = 0;
    node.child_base = child_base;
    node.tri_base = tri_base;
    uint32_t tri_off = 0, next_internal = 0;
    const double org[3] = { (double)blo[0], (double)blo[1], (double)blo[2] };
    for(int s = 0; s < 8; ++s)
    {
        const int k = w.in_slot[s];
        if(k < 0)
        {
            node.meta[s] = 0;
            node.qlo_x[s] = node.qlo_y[s] = node.qlo_z[s] = 0;
            node.qhi_x[s] = node.qhi_y[s] = node.qhi_z[s] = 0;
            continue;
        }
        const uint32_t m = static_cast<uint32_t>(w.kid[k]);
        const float4 l = nlo[m], h = nhi[m];
        const float cl[3] = { l.x, l.y, l.z }, ch[3] = { h.x, h.y, h.z };
        uint8_t ql[3], qh[3];
        for(int a = 0; a < 3; ++a)
        {
            // exact in double: the scale is a power of two
            const double sc = ldexp(1.0, ex[a]);
            double lq = floor(((double)cl[a] - org[a]) / sc);
            double hq = ceil(((double)ch[a] - org[a]) / sc);
            lq = fmax(0.0, fmin(255.0, lq));
            hq = fmax(0.0, fmin(255.0, hq));
            ql[a] = static_cast<uint8_t>(lq);
            qh[a] = static_cast<uint8_t>(hq);
        }
        node.qlo_x[s] = ql[0]; node.qlo_y[s] = ql[1]; node.qlo_z[s] = ql[2];
        node.qhi_x[s] = qh[0]; node.qhi_y[s] = qh[1]; node.qhi_z[s] = qh[2];
        if(!T.as_leaf[m])
        {
            node.imask |= static_cast<uint8_t>(1u << s);
            node.meta[s] = static_cast<uint8_t>((1u << 5) | (24u + s));
            next_level[cbase[i] + next_internal++] = m;
        }
        else
        {
            // the subtree's triangles, left to right (at most three leaves)
            uint32_t st[8];
            int sp = 0;
            st[sp++] = m;
            uint32_t cnt = 0;
            while(sp > 0)
            {
                const uint32_t x = st[--sp];
                const float4 xl = nlo[x], xh = nhi[x];
                if(f2i(xl.w) < 0)
                {
                    if(cnt >= MAX_LEAF_TRIS || tri_off + cnt >= w.n_tris)
                    {
                        atomicOr(err, 8u);
                        break;
                    }
                    out_tris[tri_base + tri_off + cnt] = tris[static_cast<uint32_t>(f2i(xh.w))];
                    ++cnt;
                }
                else if(sp + 2 <= 8)
                {
                    st[sp++] = static_cast<uint32_t>(f2i(xh.w));
                    st[sp++] = static_cast<uint32_t>(f2i(xl.w));
                }
                else
                {
                    atomicOr(err, 8u);
                    break;
                }
            }
            // triangle count in unary (1, 3, 7) above the offset
            node.meta[s] = static_cast<uint8_t>((((1u << cnt) - 1u) << 5) | tri_off);
            tri_off += cnt;
        }
    }
    out_nodes[level_base + i] = node;
}

unsigned grid_of(uint64_t n) { return static_cast<unsigned>(std::max<uint64_t>(1, (n + BLOCK - 1) / BLOCK)); }

// stream-ordered temporaries, released together
struct Temps
{
    cudaStream_t st;
    std::vector<void *> ptrs;
    cudaError_t e = cudaSuccess;
    template<class T>
    T *get(size_t count)
    {
        void *p = nullptr;
        if(e == cudaSuccess)
            e = cudaMallocAsync(&p, std::max<size_t>(1, count * sizeof(T)), st);
        if(e != cudaSuccess)
            return nullptr;
        ptrs.push_back(p);
        return static_cast<T *>(p);
    }
    ~Temps()
    {
        for(void *p : ptrs)
            cudaFreeAsync(p, st);
    }
};

} // namespace

GpuBvhStatus gpu_build_cwbvh(const TriRec *d_tris, uint32_t n, cudaStream_t st, GpuBvh &out, std::string &msg)
{
    out = GpuBvh{};
    if(n == 0)
        return GpuBvhStatus::ok;
    auto fail = [&](cudaError_t e, const char *what) {
        msg = std::string(what) + ": " + cudaGetErrorString(e);
        return GpuBvhStatus::cuda;
    };
    GpuBvhStatus status = GpuBvhStatus::ok;
    CWNode *wide = nullptr;
    TriRec *leaf_tris = nullptr;
    {
        Temps tmp{ st };
        const size_t nb = 2 * static_cast<size_t>(n) - 1;
        uint32_t *cb = tmp.get<uint32_t>(6);
        uint64_t *keys = tmp.get<uint64_t>(n), *keys2 = tmp.get<uint64_t>(n);
        uint32_t *vals = tmp.get<uint32_t>(n), *perm = tmp.get<uint32_t>(n);
        float4 *nlo = tmp.get<float4>(nb), *nhi = tmp.get<float4>(nb);
        int32_t *parent = tmp.get<int32_t>(nb);
        uint32_t *cid[2] = { tmp.get<uint32_t>(n), tmp.get<uint32_t>(n) };
        float4 *clo[2] = { tmp.get<float4>(n), tmp.get<float4>(n) };
        float4 *chi[2] = { tmp.get<float4>(n), tmp.get<float4>(n) };
        uint32_t *nn = tmp.get<uint32_t>(n);
        uint32_t *keep = tmp.get<uint32_t>(static_cast<size_t>(n) + 1);
        uint32_t *pos = tmp.get<uint32_t>(static_cast<size_t>(n) + 1);
        uint32_t *counters = tmp.get<uint32_t>(4);  // merge slot, error flags
        if(tmp.e != cudaSuccess)
            return fail(tmp.e, "device BVH temporaries");

        size_t sort_bytes = 0, scan_bytes = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, keys, keys2, vals, perm, static_cast<int>(n), 0, 63, st);
        cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, keep, pos, static_cast<int>(n) + 1, st);
        void *cub_tmp = tmp.get<uint8_t>(std::max(sort_bytes, scan_bytes));
        if(tmp.e != cudaSuccess)
            return fail(tmp.e, "device BVH temporaries");

        cudaError_t e = cudaMemsetAsync(cb, 0xff, 3 * sizeof(uint32_t), st);
        if(e == cudaSuccess)
            e = cudaMemsetAsync(cb + 3, 0, 3 * sizeof(uint32_t), st);
        if(e == cudaSuccess)
            e = cudaMemsetAsync(counters, 0, 4 * sizeof(uint32_t), st);
        if(e == cudaSuccess)
            e = cudaMemsetAsync(parent, 0xff, nb * sizeof(int32_t), st);
        if(e != cudaSuccess)
            return fail(e, "device BVH clear");
        k_centroid_bounds<<<std::min(grid_of(n), 152u * 8u), BLOCK, 0, st>>>(d_tris, n, cb);
        k_morton<<<grid_of(n), BLOCK, 0, st>>>(d_tris, n, cb, keys, vals);
        e = cub::DeviceRadixSort::SortPairs(cub_tmp, sort_bytes, keys, keys2, vals, perm, static_cast<int>(n), 0, 63,
                                            st);
        if(e != cudaSuccess)
            return fail(e, "Morton sort");
        k_leaves<<<grid_of(n), BLOCK, 0, st>>>(d_tris, perm, n, nlo, nhi, cid[0], clo[0], chi[0]);
        if((e = cudaGetLastError()) != cudaSuccess)
            return fail(e, "device BVH leaves");

        // clustering: nearest neighbours, merges of mutual pairs, compaction
        uint32_t m = n;
        int cur = 0, iterations = 0;
        // small readbacks into host variables (no pinned allocation per build: concurrent
        // builds of a batch would wait on each other's page-locking)
        uint32_t h_m_value = 0;
        uint32_t *h_m = &h_m_value;
        while(m > 1)
        {
            if(++iterations > MAX_ITERATIONS)
            {
                status = GpuBvhStatus::no_progress;
                break;
            }
            k_nearest<<<grid_of(m), BLOCK, 0, st>>>(m, clo[cur], chi[cur], nn);
            k_merge<<<grid_of(m), BLOCK, 0, st>>>(m, n, nn, cid[cur], clo[cur], chi[cur], nlo, nhi, parent, counters,
                                                  keep, counters + 1);
            e = cub::DeviceScan::ExclusiveSum(cub_tmp, scan_bytes, keep, pos, static_cast<int>(m) + 1, st);
            if(e != cudaSuccess)
                break;
            k_compact<<<grid_of(m), BLOCK, 0, st>>>(m, keep, pos, cid[cur], clo[cur], chi[cur], cid[cur ^ 1],
                                                    clo[cur ^ 1], chi[cur ^ 1]);
            cur ^= 1;
            if((e = cudaMemcpyAsync(h_m, pos + m, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
               (e = cudaStreamSynchronize(st)) != cudaSuccess)
                break;
            const uint32_t next = *h_m;
            if(next >= m || next == 0)
            {
                status = GpuBvhStatus::no_progress;
                break;
            }
            m = next;
        }
        if(e != cudaSuccess)
            return fail(e, "device BVH clustering");
        if(status != GpuBvhStatus::ok)
        {
            msg = "device BVH clustering stopped merging";
            return status;
        }
        out.ploc_iterations = iterations;
        out.binary_nodes = static_cast<uint32_t>(nb);
        uint32_t root = 0;
        if((e = cudaMemcpyAsync(&root, cid[cur], sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
           (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return fail(e, "device BVH root");
        if(n > 1 && root != nb - 1)
        {
            msg = "device BVH clustering left an incomplete tree";
            return GpuBvhStatus::internal;
        }

        // collapse tables bottom-up
        Tables T;
        T.cost = tmp.get<float>(nb * 8);
        T.split = tmp.get<uint8_t>(nb * 8);
        T.split8 = tmp.get<uint8_t>(nb);
        T.as_leaf = tmp.get<uint8_t>(nb);
        T.ntri = tmp.get<uint32_t>(nb);
        uint32_t *visits = tmp.get<uint32_t>(n);
        if(tmp.e != cudaSuccess)
            return fail(tmp.e, "device BVH tables");
        if((e = cudaMemsetAsync(visits, 0, sizeof(uint32_t) * n, st)) != cudaSuccess)
            return fail(e, "device BVH clear");
        k_collapse<<<grid_of(n), BLOCK, 0, st>>>(n, nlo, nhi, parent, visits, T);

        // emission, level by level; at most one wide node per binary node
        const uint32_t node_cap = n;
        CWNode *nodes_tmp = tmp.get<CWNode>(node_cap);
        if(cudaMalloc(&leaf_tris, sizeof(TriRec) * n) != cudaSuccess)
        {
            cudaGetLastError();
            leaf_tris = nullptr;
            return fail(cudaErrorMemoryAllocation, "device BVH triangles");
        }
        uint32_t *level[2] = { tmp.get<uint32_t>(n), tmp.get<uint32_t>(n) };
        KidSet *kids = tmp.get<KidSet>(n);
        uint32_t *ni = tmp.get<uint32_t>(static_cast<size_t>(n) + 1), *nt = tmp.get<uint32_t>(static_cast<size_t>(n) + 1);
        uint32_t *cbase = tmp.get<uint32_t>(static_cast<size_t>(n) + 1);
        uint32_t *tbase = tmp.get<uint32_t>(static_cast<size_t>(n) + 1);
        uint32_t totals[4] = {};
        if(tmp.e != cudaSuccess)
        {
            cudaFree(leaf_tris);
            leaf_tris = nullptr;
            return fail(tmp.e, "device BVH emission buffers");
        }
        e = cudaMemcpyAsync(level[0], &root, sizeof(uint32_t), cudaMemcpyHostToDevice, st);
        uint32_t count = 1, level_base = 0, tri_cursor = 0;
        int lv = 0, depth = 0;
        while(e == cudaSuccess && count > 0)
        {
            if(++depth > TRAVERSAL_STACK_SIZE)
            {
                status = GpuBvhStatus::too_deep;
                break;
            }
            k_kids<<<grid_of(count), BLOCK, 0, st>>>(level[lv], count, nlo, nhi, T, kids, ni, nt, counters + 1);
            if((e = cub::DeviceScan::ExclusiveSum(cub_tmp, scan_bytes, ni, cbase, static_cast<int>(count) + 1, st)) !=
                   cudaSuccess ||
               (e = cub::DeviceScan::ExclusiveSum(cub_tmp, scan_bytes, nt, tbase, static_cast<int>(count) + 1, st)) !=
                   cudaSuccess)
                break;
            if((e = cudaMemcpyAsync(totals, cbase + count, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) !=
                   cudaSuccess ||
               (e = cudaMemcpyAsync(totals + 1, tbase + count, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) !=
                   cudaSuccess ||
               (e = cudaMemcpyAsync(totals + 2, counters + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) !=
                   cudaSuccess ||
               (e = cudaStreamSynchronize(st)) != cudaSuccess)
                break;
            const uint32_t next_base = level_base + count;
            if(totals[2] != 0 || static_cast<uint64_t>(next_base) + totals[0] > node_cap ||
               static_cast<uint64_t>(tri_cursor) + totals[1] > n)
            {
                status = GpuBvhStatus::internal;
                break;
            }
            k_emit<<<grid_of(count), BLOCK, 0, st>>>(level[lv], count, kids, cbase, tbase, level_base, next_base,
                                                     tri_cursor, nlo, nhi, T, d_tris, n, nodes_tmp, node_cap,
                                                     leaf_tris, level[lv ^ 1], counters + 1);
            if((e = cudaGetLastError()) != cudaSuccess)
                break;
            lv ^= 1;
            level_base = next_base;
            tri_cursor += totals[1];
            count = totals[0];
        }
        if(e == cudaSuccess && status == GpuBvhStatus::ok)
        {
            // the last level's range checks
            if((e = cudaMemcpyAsync(totals + 2, counters + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) ==
                   cudaSuccess &&
               (e = cudaStreamSynchronize(st)) == cudaSuccess && (totals[2] != 0 || tri_cursor != n))
                status = GpuBvhStatus::internal;
        }
        if(e == cudaSuccess && status == GpuBvhStatus::ok)
        {
            if(cudaMalloc(&wide, sizeof(CWNode) * level_base) != cudaSuccess)
            {
                cudaGetLastError();
                wide = nullptr;
                e = cudaErrorMemoryAllocation;
            }
            else
                e = cudaMemcpyAsync(wide, nodes_tmp, sizeof(CWNode) * level_base, cudaMemcpyDeviceToDevice, st);
        }
        if(e != cudaSuccess || status != GpuBvhStatus::ok)
        {
            cudaFree(leaf_tris);
            cudaFree(wide);
            if(e != cudaSuccess)
                return fail(e, "device BVH emission");
            msg = status == GpuBvhStatus::too_deep ? "device BVH deeper than the traversal stack"
                                                   : "device BVH emission failed a range check";
            return status;
        }
        out.node_count = level_base;
        out.depth = depth;
    }
    // the temporaries are released on the stream; the result is complete once it drains
    const cudaError_t e = cudaStreamSynchronize(st);
    if(e != cudaSuccess)
    {
        cudaFree(leaf_tris);
        cudaFree(wide);
        return fail(e, "device BVH build");
    }
    out.nodes = wide;
    out.tris = leaf_tris;
    out.tri_count = n;
    return GpuBvhStatus::ok;
}

} // namespace bt
