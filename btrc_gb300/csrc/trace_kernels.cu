// Ray-batch traversal kernels behind btrc_trace_closest / btrc_trace_any: the
// replacement for the reference's OptiX trace and shadow launches
// (builtin/btrc/builtin/renderer/wavefront/trace.cpp:38-78, shadow.cpp:24-76).
#include "kernels.h"
#include "traverse.cuh"
#include "two_level.cuh"

namespace bt {

namespace {

constexpr int TRACE_BLOCK = TRAVERSE_BLOCK;  // traverse_refill's shared-memory slices

__global__ void __launch_bounds__(TRACE_BLOCK) k_trace_stats(DevScene S, const Ray *__restrict__ rays, uint32_t n,
                                                             uint32_t *__restrict__ nv, uint32_t *__restrict__ tv,
                                                             uint32_t *err)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        const float4 ro = __ldg(reinterpret_cast<const float4 *>(rays) + i * 2);
        const float4 rd = __ldg(reinterpret_cast<const float4 *>(rays) + i * 2 + 1);
        const TravRay tr = make_trav_ray(ro.x, ro.y, ro.z, rd.x, rd.y, rd.z);
        uint32_t a = 0, b = 0;
        trace_closest(tr, rd.w, reinterpret_cast<const float4 *>(S.nodes), reinterpret_cast<const float4 *>(S.tris),
                      S.node_count, err, &a, &b);
        nv[i] = a;
        tv[i] = b;
    }
}

// persistent kernels with warp-level ray refill (traverse_refill); the cursor must be
// zero at launch
__global__ void __launch_bounds__(TRACE_BLOCK) k_trace_closest_dyn(DevScene S, const Ray *__restrict__ rays, uint32_t n,
                                                                   uint32_t *__restrict__ flags,
                                                                   HitDetail *__restrict__ hits, uint32_t *cursor,
                                                                   uint32_t *err)
{
    traverse_refill<false>(
        reinterpret_cast<const float4 *>(S.nodes), reinterpret_cast<const float4 *>(S.tris), S.node_count, cursor, n,
        REFILL_LANES, err,
        [&](uint32_t i, float *o, float *d, float &t1, uint32_t &) {
            const float4 ro = __ldg(reinterpret_cast<const float4 *>(rays) + i * 2);
            const float4 rd = __ldg(reinterpret_cast<const float4 *>(rays) + i * 2 + 1);
            o[0] = ro.x; o[1] = ro.y; o[2] = ro.z;
            d[0] = rd.x; d[1] = rd.y; d[2] = rd.z;
            t1 = rd.w;
        },
        [&](uint32_t i, const ClosestResult &c) {
            flags[i] = c.hit ? (c.inst | HIT_BIT) : 0u;
            hits[i] = c.hit ? HitDetail{ c.t, c.prim, c.b1, c.b2 } : HitDetail{ 0.0f, 0u, 0.0f, 0.0f };
        },
        nullptr, nullptr, S.tri_round);
}

__global__ void __launch_bounds__(TRACE_BLOCK) k_trace_any_dyn(DevScene S, const Ray *__restrict__ rays, uint32_t n,
                                                               uint32_t *__restrict__ occluded, uint32_t *cursor,
                                                               uint32_t *err)
{
    traverse_refill<true>(
        reinterpret_cast<const float4 *>(S.nodes), reinterpret_cast<const float4 *>(S.tris), S.node_count, cursor, n,
        REFILL_LANES, err,
        [&](uint32_t i, float *o, float *d, float &t1, uint32_t &) {
            const float4 ro = __ldg(reinterpret_cast<const float4 *>(rays) + i * 2);
            const float4 rd = __ldg(reinterpret_cast<const float4 *>(rays) + i * 2 + 1);
            o[0] = ro.x; o[1] = ro.y; o[2] = ro.z;
            d[0] = rd.x; d[1] = rd.y; d[2] = rd.z;
            t1 = rd.w;
        },
        [&](uint32_t i, const ClosestResult &c) { occluded[i] = c.hit ? 1u : 0u; }, nullptr, nullptr,
        S.shadow_round);
}

// the two-level form (the cursor must be zero at launch)
template<bool ANY>
__global__ void __launch_bounds__(TRACE_BLOCK) k_trace_two_level(DevScene S, const Ray *__restrict__ rays, uint32_t n,
                                                                 uint32_t *__restrict__ flags,
                                                                 HitDetail *__restrict__ hits,
                                                                 uint32_t *__restrict__ occluded, uint32_t *cursor,
                                                                 uint32_t *err)
{
    traverse_refill<ANY, false, true>(
        reinterpret_cast<const float4 *>(S.nodes), reinterpret_cast<const float4 *>(S.tris), S.node_count, cursor, n,
        REFILL_LANES, err,
        [&](uint32_t i, float *o, float *d, float &t1, uint32_t &) {
            const float4 ro = __ldg(reinterpret_cast<const float4 *>(rays) + i * 2);
            const float4 rd = __ldg(reinterpret_cast<const float4 *>(rays) + i * 2 + 1);
            o[0] = ro.x; o[1] = ro.y; o[2] = ro.z;
            d[0] = rd.x; d[1] = rd.y; d[2] = rd.z;
            t1 = rd.w;
        },
        [&](uint32_t i, const ClosestResult &c) {
            if(ANY)
                occluded[i] = c.hit ? 1u : 0u;
            else
            {
                flags[i] = c.hit ? (c.inst | HIT_BIT) : 0u;
                hits[i] = c.hit ? HitDetail{ c.t, c.prim, c.b1, c.b2 } : HitDetail{ 0.0f, 0u, 0.0f, 0.0f };
            }
        },
        nullptr, nullptr, ANY ? S.shadow_round : S.tri_round, two_level_view(S));
}

uint32_t persistent_blocks(const void *kernel)
{
    int dev = 0, sms = 152, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, TRACE_BLOCK, 0);
    return static_cast<uint32_t>(sms * (per_sm > 0 ? per_sm : 1));
}

uint32_t grid_for(uint32_t n, int block)
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t want = (static_cast<uint64_t>(n) + block - 1) / block;
    const uint64_t cap = static_cast<uint64_t>(sms) * 16;
    return static_cast<uint32_t>(want < cap ? (want > 0 ? want : 1) : cap);
}

} // namespace

cudaError_t launch_trace_closest(const DevScene &S, const Ray *rays, uint32_t n, uint32_t *flags, HitDetail *hits,
                                 uint32_t *err, cudaStream_t st)
{
    if(n == 0)
        return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(err + 4, 0, sizeof(uint32_t), st);
    if(e != cudaSuccess)
        return e;
    if(S.two_level)
    {
        k_trace_two_level<false>
            <<<persistent_blocks(reinterpret_cast<const void *>(k_trace_two_level<false>)), TRACE_BLOCK, 0, st>>>(
                S, rays, n, flags, hits, nullptr, err + 4, err);
        return cudaGetLastError();
    }
    k_trace_closest_dyn<<<persistent_blocks(reinterpret_cast<const void *>(k_trace_closest_dyn)), TRACE_BLOCK, 0, st>>>(
        S, rays, n, flags, hits, err + 4, err);
    return cudaGetLastError();
}

cudaError_t launch_trace_any(const DevScene &S, const Ray *rays, uint32_t n, uint32_t *occluded, uint32_t *err,
                             cudaStream_t st)
{
    if(n == 0)
        return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(err + 8, 0, sizeof(uint32_t), st);
    if(e != cudaSuccess)
        return e;
    if(S.two_level)
    {
        k_trace_two_level<true>
            <<<persistent_blocks(reinterpret_cast<const void *>(k_trace_two_level<true>)), TRACE_BLOCK, 0, st>>>(
                S, rays, n, nullptr, nullptr, occluded, err + 8, err);
        return cudaGetLastError();
    }
    k_trace_any_dyn<<<persistent_blocks(reinterpret_cast<const void *>(k_trace_any_dyn)), TRACE_BLOCK, 0, st>>>(
        S, rays, n, occluded, err + 8, err);
    return cudaGetLastError();
}

cudaError_t launch_trace_stats(const DevScene &S, const Ray *rays, uint32_t n, uint32_t *nv, uint32_t *tv,
                               uint32_t *err, cudaStream_t st)
{
    if(n == 0)
        return cudaSuccess;
    if(S.two_level)
        return cudaErrorNotSupported;  // node / triangle counts are kept for the single-level form
    k_trace_stats<<<grid_for(n, TRACE_BLOCK), TRACE_BLOCK, 0, st>>>(S, rays, n, nv, tv, err);
    return cudaGetLastError();
}

} // namespace bt
