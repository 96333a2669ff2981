// Host BVH builder: binned SAH over world-space triangles (SAH cost accumulated in
// FP64), built by fork-join tasks on all host cores, collapsed into an 8-wide tree whose child boxes are quantised to 8 bits
// relative to a per-node origin and power-of-two scale (80-byte nodes, 16-byte aligned).
// This replaces the OptiX GAS/IAS build the reference calls
// (common/btrc/utils/optix/context.cpp:106-215).
#pragma once

#include <vector>

#include "layout.h"
#include "taskpool.h"

namespace bt {

struct CWBVH
{
    std::vector<CWNode> nodes;
    std::vector<TriRec> tris;   // leaf order
    int depth = 0;              // number of wide levels
    int binary_nodes = 0;
};

// Wide levels the traversal stack can hold; the builder refuses deeper trees.
constexpr int TRAVERSAL_STACK_SIZE = 32;

// tris: world-space triangles with inst/prim ids. threads <= 0 means hardware concurrency.
// The result depends only on the triangles, not on the thread count.
CWBVH build_cwbvh(const std::vector<TriRec> &tris, int threads);
// the same on the threads of an existing task pool
CWBVH build_cwbvh(const std::vector<TriRec> &tris, TaskPool &pool);

} // namespace bt
