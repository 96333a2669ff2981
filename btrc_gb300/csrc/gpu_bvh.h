// Device BVH builder: the same 8-wide compressed layout as the host builder (bvh.h),
// built on the GPU for scenes whose build would otherwise dominate their render (batches
// of many scenes, cold starts). The binary tree comes from PLOC (Meister and Bittner,
// "Parallel locally-ordered clustering for bounding volume hierarchy construction",
// IEEE TVCG 2018) over 63-bit Morton order; the 8-wide collapse is the host builder's
// dynamic programme (Ylitie, Karras and Laine 2017), run bottom-up on the device, and the
// nodes are emitted level by level in the host builder's breadth-first layout. This
// replaces the OptiX GAS/IAS build the reference calls
// (common/btrc/utils/optix/context.cpp:106-215) where build time matters more than the
// last few per cent of traversal speed.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "layout.h"

namespace bt {

struct GpuBvh
{
    CWNode *nodes = nullptr;  // cudaMalloc'd, owned by the caller
    TriRec *tris = nullptr;   // leaf order, cudaMalloc'd, owned by the caller
    uint32_t node_count = 0;
    uint32_t tri_count = 0;
    int depth = 0;            // wide levels
    uint32_t binary_nodes = 0;
    int ploc_iterations = 0;
};

enum class GpuBvhStatus
{
    ok,
    cuda,         // a CUDA call failed (message set)
    no_progress,  // the clustering stopped merging (non-finite boxes); build on the host
    too_deep,     // more wide levels than the traversal stack holds; build on the host
    internal      // a device-side range check failed (message set)
};

// d_tris: n world-space triangles in device memory. Runs on `stream` and returns after
// the stream has finished; temporaries come from the stream-ordered allocator.
GpuBvhStatus gpu_build_cwbvh(const TriRec *d_tris, uint32_t n, cudaStream_t stream, GpuBvh &out, std::string &msg);

} // namespace bt
