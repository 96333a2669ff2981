// Ray-batch traversal kernels behind btrc_trace_closest / btrc_trace_any: the
// replacement for the reference's OptiX trace and shadow launches
// (builtin/btrc/builtin/renderer/wavefront/trace.cpp:38-78, shadow.cpp:24-76).
#include "kernels.h"
#include "traverse.cuh"

namespace bt {

namespace {

constexpr int TRACE_BLOCK = 128;

__global__ void __launch_bounds__(TRACE_BLOCK) k_trace_closest(DevScene S, const Ray *__restrict__ rays, uint32_t n,
                                                               uint32_t *__restrict__ flags,
                                                               HitDetail *__restrict__ hits, uint32_t *err)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        const float4 ro = __ldg(reinterpret_cast<const float4 *>(rays) + i * 2);
        const float4 rd = __ldg(reinterpret_cast<const float4 *>(rays) + i * 2 + 1);
        const TravRay tr = make_trav_ray(ro.x, ro.y, ro.z, rd.x, rd.y, rd.z);
        const ClosestResult c = trace_closest(tr, rd.w, reinterpret_cast<const float4 *>(S.nodes),
                                              reinterpret_cast<const float4 *>(S.tris), S.node_count, err);
        if(c.hit)
        {
            flags[i] = c.inst | HIT_BIT;
            hits[i] = HitDetail{ c.t, c.prim, c.b1, c.b2 };
        }
        else
        {
            flags[i] = 0u;
            hits[i] = HitDetail{ 0.0f, 0u, 0.0f, 0.0f };
        }
    }
}

__global__ void __launch_bounds__(TRACE_BLOCK) k_trace_any(DevScene S, const Ray *__restrict__ rays, uint32_t n,
                                                           uint32_t *__restrict__ occluded, uint32_t *err)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        const float4 ro = __ldg(reinterpret_cast<const float4 *>(rays) + i * 2);
        const float4 rd = __ldg(reinterpret_cast<const float4 *>(rays) + i * 2 + 1);
        const TravRay tr = make_trav_ray(ro.x, ro.y, ro.z, rd.x, rd.y, rd.z);
        occluded[i] = trace_any(tr, rd.w, reinterpret_cast<const float4 *>(S.nodes),
                                reinterpret_cast<const float4 *>(S.tris), S.node_count, err) ? 1u : 0u;
    }
}

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
    k_trace_closest<<<grid_for(n, TRACE_BLOCK), TRACE_BLOCK, 0, st>>>(S, rays, n, flags, hits, err);
    return cudaGetLastError();
}

cudaError_t launch_trace_any(const DevScene &S, const Ray *rays, uint32_t n, uint32_t *occluded, uint32_t *err,
                             cudaStream_t st)
{
    if(n == 0)
        return cudaSuccess;
    k_trace_any<<<grid_for(n, TRACE_BLOCK), TRACE_BLOCK, 0, st>>>(S, rays, n, occluded, err);
    return cudaGetLastError();
}

cudaError_t launch_trace_stats(const DevScene &S, const Ray *rays, uint32_t n, uint32_t *nv, uint32_t *tv,
                               uint32_t *err, cudaStream_t st)
{
    if(n == 0)
        return cudaSuccess;
    k_trace_stats<<<grid_for(n, TRACE_BLOCK), TRACE_BLOCK, 0, st>>>(S, rays, n, nv, tv, err);
    return cudaGetLastError();
}

} // namespace bt
