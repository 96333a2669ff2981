// ORACLE — test infrastructure only. Thin C driver over the BVH library vendored in the
// reference tree (lib/bvh, madmann91/bvh, header-only, used by the reference at
// src/core/btrc/core/volume/bvh.cpp:56-63). It is compiled from those headers where they
// lie (oracle/build.py) into oracle/_ref/ and serves two purposes: a reference answer for
// closest-hit traversal on identical ray batches, and the CPU traversal baseline.
// Its triangle test is not watertight, so agreement with the watertight kernels is
// expected everywhere except on rays that graze shared edges.
#include <cstdint>
#include <vector>

#include <bvh/bvh.hpp>
#include <bvh/primitive_intersectors.hpp>
#include <bvh/ray.hpp>
#include <bvh/single_ray_traverser.hpp>
#include <bvh/sweep_sah_builder.hpp>
#include <bvh/triangle.hpp>
#include <bvh/vector.hpp>

using Scalar = float;
using Vec = bvh::Vector3<Scalar>;
using Tri = bvh::Triangle<Scalar>;
using Ray = bvh::Ray<Scalar>;
using Bvh = bvh::Bvh<Scalar>;

struct RefScene
{
    std::vector<Tri> tris;
    Bvh bvh;
};

extern "C" {

void *ref_build(const float *xyz, uint64_t n)
{
    auto *s = new RefScene();
    s->tris.reserve(n);
    for(uint64_t i = 0; i < n; ++i)
    {
        const float *p = xyz + i * 9;
        s->tris.emplace_back(Vec(p[0], p[1], p[2]), Vec(p[3], p[4], p[5]), Vec(p[6], p[7], p[8]));
    }
    auto [boxes, centers] = bvh::compute_bounding_boxes_and_centers(s->tris.data(), s->tris.size());
    auto global = bvh::compute_bounding_boxes_union(boxes.get(), s->tris.size());
    bvh::SweepSahBuilder<Bvh> builder(s->bvh);
    builder.build(global, boxes.get(), centers.get(), s->tris.size());
    return s;
}

void ref_free(void *s) { delete static_cast<RefScene *>(s); }

// rays: 8 floats (o.xyz, pad, d.xyz, t1). prim = -1 on a miss.
void ref_closest(const void *sp, const float *rays, uint64_t m, int64_t *prim, float *t)
{
    const RefScene &s = *static_cast<const RefScene *>(sp);
    bvh::ClosestPrimitiveIntersector<Bvh, Tri> isect(s.bvh, s.tris.data());
    bvh::SingleRayTraverser<Bvh> trav(s.bvh);
#pragma omp parallel for schedule(dynamic, 256)
    for(int64_t i = 0; i < static_cast<int64_t>(m); ++i)
    {
        const float *r = rays + i * 8;
        Ray ray(Vec(r[0], r[1], r[2]), Vec(r[4], r[5], r[6]), 0.0f, r[7]);
        if(auto hit = trav.traverse(ray, isect))
        {
            prim[i] = static_cast<int64_t>(hit->primitive_index);
            t[i] = hit->intersection.t;
        }
        else
        {
            prim[i] = -1;
            t[i] = 0.0f;
        }
    }
}

} // extern "C"
