// C-ABI implementation: host runtime around the CUDA kernels. No C++ exception
// crosses this boundary; every failure becomes a btrc_status plus a message.
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <memory>
#include <mutex>
#include <new>
#include <numeric>
#include <map>
#include <set>
#include <thread>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "btrc.h"
#include "bvh.h"
#include "gpu_bvh.h"
#include "image_io.h"
#include "nrc.h"
#include "kernels.h"
#include "scene.h"

using namespace bt;

// One render lane of the batch renderer: its own stream, queues, film and scratch.
struct BatchLane
{
    cudaStream_t stream = nullptr;
    RenderBuffers buf{};
    std::vector<void *> allocs;
    uint32_t capacity = 0;
    size_t pixels = 0;
    float *rgb = nullptr;      // device image for host outputs
    size_t rgb_pixels = 0;
    uint32_t *err = nullptr;
    ~BatchLane();
};

// A merged batch: several built scenes concatenated into one device scene (see
// merge_scenes), their per-scene table and the combined film's shape.
struct MergedBatch
{
    std::vector<const btrc_scene *> scenes;
    std::vector<uint64_t> serials;
    std::vector<void *> allocs;
    DevScene S{};
    std::vector<BatchScene> table;   // in queue order: fewest camera paths first
    std::vector<uint32_t> input;     // table entry -> position in the caller's scene list
    BatchScene *d_table = nullptr;
    uint8_t *d_row_scene = nullptr;
    BatchOut *d_outs = nullptr;
    uint32_t film_width = 0, film_rows = 0;
    uint64_t total_paths = 0;
    int min_depth = 0, max_depth = 0;
    // autotuner's choice for this batch
    bool tuned = false;
    uint32_t capacity = 0;
    int block = 0, grid_pct = 100;
    ~MergedBatch()
    {
        for(void *p : allocs)
            cudaFree(p);
    }
};

struct btrc_ctx
{
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    std::atomic<bool> cancel{ false };
    // render buffers, grown on demand and reused across renders
    RenderBuffers buf{};
    std::vector<void *> buf_allocs;
    uint32_t buf_capacity = 0;
    size_t film_pixels = 0;
    bool has_media_buffers = false;
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    float *denoise_tmp = nullptr;  // ping-pong image of the denoise post-processor
    size_t denoise_bytes = 0;
    std::set<btrc_scene *> scenes;  // live scenes, destroyed with the context
    // batched rendering: concurrent lanes and the autotuner's choices per scene class
    std::vector<std::unique_ptr<struct BatchLane>> lanes;
    std::map<std::pair<int, int>, std::pair<uint32_t, int>> tuned;  // (pixel class, triangle class) -> (capacity, grid %)
    std::unique_ptr<MergedBatch> merged;                              // the last merged batch of scenes
    // radiance-cache frame buffers (queries, weights, predictions, training samples)
    std::vector<void *> nrc_allocs;
    size_t nrc_pixels = 0;
    float *nrc_query = nullptr;
    float4 *nrc_weight = nullptr, *nrc_pred = nullptr;
    uint32_t *nrc_counts = nullptr;
    float2 *nrc_spread[2] = {};      // path-spread state per queue slot, by bounce parity
};

struct btrc_scene
{
    btrc_ctx *ctx = nullptr;
    HostScene host;
    bool built = false;
    DevScene dev{};
    std::vector<void *> allocs;
    int bvh_nodes = 0, bvh_depth = 0;
    uint64_t bvh_bytes = 0;
    double build_ms = 0;
    double bvh_ms = 0;
    int bvh_builder = 0;             // 0 host, 1 device
    bool two_level = false;          // per-geometry trees under a top level over instances
    std::vector<AliasEntry8> filter_table_host;
    AliasEntry8 *filter_table = nullptr;
    uint64_t export_count = 0;       // flattened triangles (btrc_scene_export_triangles)
    std::vector<CWNode> host_nodes;  // kept for host-only contexts and small scenes
    std::vector<TriRec> host_tris;
    uint64_t n_shade_tris = 0;       // shading records (triangles over all geometries)
    uint64_t n_light_tris = 0;       // triangles of light geometries (light sampling arrays)
    uint64_t serial = 0;             // build number, for caches built from this scene
};

namespace {

struct StatusError : std::runtime_error
{
    btrc_status status;
    StatusError(btrc_status s, const std::string &m) : std::runtime_error(m), status(s) {}
};

void check_cuda(cudaError_t e, const char *what)
{
    if(e == cudaSuccess)
        return;
    const btrc_status s = e == cudaErrorMemoryAllocation ? BTRC_ERR_OOM : BTRC_ERR_CUDA;
    throw StatusError(s, std::string(what) + ": " + cudaGetErrorString(e));
}

template<typename F>
btrc_status guarded(btrc_ctx *ctx, F &&f)
{
    try
    {
        f();
        if(ctx)
            ctx->last_error.clear();
        return BTRC_OK;
    }
    catch(const StatusError &e)
    {
        if(ctx)
            ctx->last_error = e.what();
        return e.status;
    }
    catch(const json::ParseError &e)
    {
        if(ctx)
            ctx->last_error = e.what();
        return std::string(e.what()).find("cannot open") != std::string::npos ? BTRC_ERR_IO : BTRC_ERR_PARSE;
    }
    catch(const std::bad_alloc &)
    {
        if(ctx)
            ctx->last_error = "host allocation failed";
        return BTRC_ERR_OOM;
    }
    catch(const std::exception &e)
    {
        if(ctx)
            ctx->last_error = e.what();
        const std::string m = e.what();
        if(m.find("cannot open") != std::string::npos || m.find("failed to open") != std::string::npos)
            return BTRC_ERR_IO;
        if(m.find("unsupported") != std::string::npos)
            return BTRC_ERR_UNSUPPORTED;
        return BTRC_ERR_PARSE;
    }
    catch(...)
    {
        if(ctx)
            ctx->last_error = "unknown internal error";
        return BTRC_ERR_INTERNAL;
    }
}

template<typename T>
T *dev_upload(std::vector<void *> &allocs, const T *src, size_t count)
{
    if(count == 0)
        return nullptr;
    void *p = nullptr;
    check_cuda(cudaMalloc(&p, sizeof(T) * count), "cudaMalloc");
    allocs.push_back(p);
    check_cuda(cudaMemcpy(p, src, sizeof(T) * count, cudaMemcpyHostToDevice), "cudaMemcpy");
    return static_cast<T *>(p);
}

void *dev_alloc(std::vector<void *> &allocs, size_t bytes)
{
    void *p = nullptr;
    check_cuda(cudaMalloc(&p, bytes > 0 ? bytes : 16), "cudaMalloc");
    allocs.push_back(p);
    return p;
}

void free_all(std::vector<void *> &allocs)
{
    for(void *p : allocs)
        cudaFree(p);
    allocs.clear();
}

void extended_gcd(uint64_t a, uint64_t b, int64_t *x, int64_t *y)
{
    if(b == 0)
    {
        *x = 1;
        *y = 0;
        return;
    }
    const int64_t d = static_cast<int64_t>(a / b);
    int64_t xp, yp;
    extended_gcd(b, a % b, &xp, &yp);
    *x = yp;
    *y = xp - d * yp;
}

int64_t mult_inverse(int64_t a, int64_t n)
{
    int64_t x, y;
    extended_gcd(static_cast<uint64_t>(a), static_cast<uint64_t>(n), &x, &y);
    int64_t r = x - x / n * n;
    return r < 0 ? r + n : r;
}

// HaltonSampler::initialize_consts (builtin/btrc/builtin/sampler/halton.cpp:140-160)
HaltonConsts halton_consts(int width, int height)
{
    HaltonConsts hc{};
    const int res[2] = { width, height };
    for(int i = 0; i < 2; ++i)
    {
        const int base = i == 0 ? 2 : 3;
        int scale = 1, e = 0;
        while(scale < std::min(res[i], HALTON_MAX_RES))
        {
            scale *= base;
            ++e;
        }
        hc.scale[i] = scale;
        hc.exponent[i] = e;
    }
    hc.mult_inverse[0] = static_cast<int32_t>(mult_inverse(hc.scale[1], hc.scale[0]));
    hc.mult_inverse[1] = static_cast<int32_t>(mult_inverse(hc.scale[0], hc.scale[1]));
    hc.stride = hc.scale[0] * hc.scale[1];
    return hc;
}

// triangle t of instance i in world space: the one transform the BVH, the oracle exports
// and the shading agree on
TriRec world_triangle(const HostScene &H, size_t i, size_t t)
{
    const HostGeometry &g = H.geometries[H.instances[i].geometry];
    const Transform &xf = H.instance_xf[i];
    const V3 a = xf.point(g.pos[t * 3 + 0]);
    const V3 b = xf.point(g.pos[t * 3 + 1]);
    const V3 c = xf.point(g.pos[t * 3 + 2]);
    return TriRec{ a.x, a.y, a.z, static_cast<uint32_t>(i), b.x, b.y, b.z, static_cast<uint32_t>(t), c.x, c.y, c.z, 0u };
}

// Two-level form: one object-space tree per geometry (host builder), a top-level tree
// over the instances' world boxes whose leaf records are the boxes themselves (v0 = low
// corner with the instance index in v0.w, v1 = high corner), so that memory grows with
// geometries, not with instances x triangles.
void build_two_level(btrc_scene *sc, TaskPool &pool, DevScene &D)
{
    const HostScene &H = sc->host;
    const size_t ng = H.geometries.size();
    std::vector<char> used(ng, 0);
    for(const auto &in : H.instances)
        used[static_cast<size_t>(in.geometry)] = 1;
    std::vector<CWNode> nodes;
    std::vector<TriRec> tris;
    std::vector<uint32_t> root(std::max<size_t>(ng, 1), 0xffffffffu);
    std::vector<std::array<float, 6>> obox(ng);
    int depth = 0;
    for(size_t g = 0; g < ng; ++g)
    {
        const HostGeometry &geo = H.geometries[g];
        const size_t nt = geo.area.size();
        if(!used[g] || nt == 0)
            continue;
        std::vector<TriRec> obj(nt);
        pool.parallel_for(nt, 1u << 14, [&](size_t b, size_t e) {
            for(size_t t = b; t < e; ++t)
            {
                const V3 a = geo.pos[t * 3 + 0], bb = geo.pos[t * 3 + 1], c = geo.pos[t * 3 + 2];
                obj[t] = TriRec{ a.x, a.y, a.z, 0u, bb.x, bb.y, bb.z, static_cast<uint32_t>(t), c.x, c.y, c.z, 0u };
            }
        });
        std::array<float, 6> bx = { MAX_FLOAT, MAX_FLOAT, MAX_FLOAT, -MAX_FLOAT, -MAX_FLOAT, -MAX_FLOAT };
        for(size_t k = 0; k < nt * 3; ++k)
        {
            const V3 &v = geo.pos[k];
            bx[0] = std::min(bx[0], v.x); bx[1] = std::min(bx[1], v.y); bx[2] = std::min(bx[2], v.z);
            bx[3] = std::max(bx[3], v.x); bx[4] = std::max(bx[4], v.y); bx[5] = std::max(bx[5], v.z);
        }
        obox[g] = bx;
        CWBVH b = build_cwbvh(obj, pool);
        const uint32_t noff = static_cast<uint32_t>(nodes.size()), toff = static_cast<uint32_t>(tris.size());
        for(CWNode &nd : b.nodes)
        {
            nd.child_base += noff;
            nd.tri_base += toff;
        }
        root[g] = noff;
        nodes.insert(nodes.end(), b.nodes.begin(), b.nodes.end());
        tris.insert(tris.end(), b.tris.begin(), b.tris.end());
        depth = std::max(depth, b.depth);
    }
    // instance boxes: the geometry box's corners through the instance transform, widened
    // by 1e-5 of the box's size and magnitude, which covers the rounding of the
    // transforms in both directions many times over
    std::vector<TriRec> boxes;
    boxes.reserve(H.instances.size());
    for(size_t i = 0; i < H.instances.size(); ++i)
    {
        const size_t g = static_cast<size_t>(H.instances[i].geometry);
        if(root[g] == 0xffffffffu)
            continue;
        const auto &bx = obox[g];
        float lo[3] = { MAX_FLOAT, MAX_FLOAT, MAX_FLOAT }, hi[3] = { -MAX_FLOAT, -MAX_FLOAT, -MAX_FLOAT };
        for(int c = 0; c < 8; ++c)
        {
            const V3 w = H.instance_xf[i].point(V3(bx[(c & 1) ? 3 : 0], bx[(c & 2) ? 4 : 1], bx[(c & 4) ? 5 : 2]));
            const float v[3] = { w.x, w.y, w.z };
            for(int a = 0; a < 3; ++a)
            {
                lo[a] = std::min(lo[a], v[a]);
                hi[a] = std::max(hi[a], v[a]);
            }
        }
        float size = 0.0f;
        for(int a = 0; a < 3; ++a)
            size = std::max(size, std::max(hi[a] - lo[a], std::max(std::fabs(lo[a]), std::fabs(hi[a]))));
        const float pad = size * 1e-5f + 1e-30f;
        for(int a = 0; a < 3; ++a)
        {
            lo[a] -= pad;
            hi[a] += pad;
        }
        boxes.push_back(TriRec{ lo[0], lo[1], lo[2], static_cast<uint32_t>(i), hi[0], hi[1], hi[2], 0u, lo[0], lo[1],
                                lo[2], 0u });
    }
    CWBVH top = build_cwbvh(boxes, pool);
    D.nodes = reinterpret_cast<const F4 *>(dev_upload(sc->allocs, top.nodes.data(), top.nodes.size()));
    D.tris = reinterpret_cast<const F4 *>(dev_upload(sc->allocs, top.tris.data(), top.tris.size()));
    D.node_count = static_cast<uint32_t>(top.nodes.size());
    D.tri_count = static_cast<uint32_t>(top.tris.size());
    D.blas_nodes = reinterpret_cast<const F4 *>(dev_upload(sc->allocs, nodes.data(), nodes.size()));
    D.blas_tris = reinterpret_cast<const F4 *>(dev_upload(sc->allocs, tris.data(), tris.size()));
    D.blas_root = dev_upload(sc->allocs, root.data(), root.size());
    D.blas_node_count = static_cast<uint32_t>(nodes.size());
    D.blas_tri_count = static_cast<uint32_t>(tris.size());
    D.instance_count = static_cast<uint32_t>(H.instances.size());
    D.two_level = 1;
    sc->bvh_nodes = static_cast<int>(top.nodes.size() + nodes.size());
    sc->bvh_depth = top.depth + depth;
    sc->bvh_bytes = (top.nodes.size() + nodes.size()) * sizeof(CWNode) + (top.tris.size() + tris.size()) * sizeof(TriRec) +
                    root.size() * sizeof(uint32_t);
    sc->two_level = true;
}

void build_scene(btrc_scene *sc, int threads, int builder, int two_level)
{
    HostScene &H = sc->host;
    const auto t0 = std::chrono::steady_clock::now();
    const bool host_only = sc->ctx->device < 0;
    if(!host_only)
    {
        check_cuda(cudaSetDevice(sc->ctx->device), "cudaSetDevice");
        free_all(sc->allocs);
    }

    if(threads <= 0)
        threads = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
    std::unique_ptr<TaskPool> own;
    TaskPool *pp = current_pool();  // a batch build's pool, else threads of our own
    if(!pp)
    {
        own = std::make_unique<TaskPool>(threads);
        pp = own.get();
    }
    TaskPool &pool = *pp;

    // flatten instances into world-space triangles (single-level BVH), in parallel over
    // triangle ranges of each instance
    std::vector<size_t> inst_first(H.instances.size() + 1, 0);
    for(size_t i = 0; i < H.instances.size(); ++i)
        inst_first[i + 1] = inst_first[i] + H.geometries[H.instances[i].geometry].area.size();
    const bool two = two_level != 0 && !host_only;
    std::vector<TriRec> world(two ? 0 : inst_first.back());
    for(size_t i = 0; i < H.instances.size() && !two; ++i)
    {
        const size_t base = inst_first[i];
        pool.parallel_for(H.geometries[H.instances[i].geometry].area.size(), 1u << 14,
                          [&, i, base](size_t tb, size_t te) {
                              for(size_t t = tb; t < te; ++t)
                                  world[base + t] = world_triangle(H, i, t);
                          });
    }
    sc->export_count = inst_first.back();
    // the traversal's pooled triangle tests address triangle records with 27 bits
    if(!host_only && !two && world.size() >= (1ull << 27))
        throw StatusError(BTRC_ERR_INVALID_ARG, "scene exceeds 2^27 triangle records");
    const bool keep_host = host_only || H.triangle_count <= (1u << 20);
    const auto tb = std::chrono::steady_clock::now();
    DevScene &D = sc->dev;
    D = DevScene{};
    sc->bvh_builder = 0;
    sc->two_level = false;
    if(two)
        build_two_level(sc, pool, D);
    else if(builder == 1 && !host_only && !world.empty())
    {
        // device build on a stream of its own, so that concurrent scene builds overlap
        cudaStream_t bst = nullptr;
        check_cuda(cudaStreamCreateWithFlags(&bst, cudaStreamNonBlocking), "build stream");
        TriRec *d_world = nullptr;
        cudaError_t e = cudaMallocAsync(&d_world, sizeof(TriRec) * world.size(), bst);
        if(e == cudaSuccess)
            e = cudaMemcpyAsync(d_world, world.data(), sizeof(TriRec) * world.size(), cudaMemcpyHostToDevice, bst);
        GpuBvh gb;
        std::string msg;
        GpuBvhStatus gs = GpuBvhStatus::cuda;
        if(e == cudaSuccess)
            gs = gpu_build_cwbvh(d_world, static_cast<uint32_t>(world.size()), bst, gb, msg);
        else
            msg = std::string("device BVH input: ") + cudaGetErrorString(e);
        cudaFreeAsync(d_world, bst);
        const cudaError_t se = cudaStreamSynchronize(bst);
        cudaStreamDestroy(bst);
        if(gs == GpuBvhStatus::ok && se == cudaSuccess)
        {
            sc->allocs.push_back(gb.nodes);
            sc->allocs.push_back(gb.tris);
            D.nodes = reinterpret_cast<const F4 *>(gb.nodes);
            D.tris = reinterpret_cast<const F4 *>(gb.tris);
            D.node_count = gb.node_count;
            D.tri_count = gb.tri_count;
            sc->bvh_nodes = static_cast<int>(gb.node_count);
            sc->bvh_depth = gb.depth;
            sc->bvh_bytes = static_cast<uint64_t>(gb.node_count) * sizeof(CWNode) + uint64_t(gb.tri_count) * sizeof(TriRec);
            sc->bvh_builder = 1;
            if(keep_host)
            {
                sc->host_nodes.resize(gb.node_count);
                sc->host_tris.resize(gb.tri_count);
                check_cuda(cudaMemcpy(sc->host_nodes.data(), gb.nodes, sizeof(CWNode) * gb.node_count,
                                      cudaMemcpyDeviceToHost),
                           "BVH download");
                check_cuda(cudaMemcpy(sc->host_tris.data(), gb.tris, sizeof(TriRec) * gb.tri_count,
                                      cudaMemcpyDeviceToHost),
                           "BVH download");
            }
        }
        else
        {
            cudaFree(gb.nodes);
            cudaFree(gb.tris);
            if(se != cudaSuccess)
                throw StatusError(BTRC_ERR_CUDA, std::string("device BVH build: ") + cudaGetErrorString(se));
            if(gs == GpuBvhStatus::cuda)
                throw StatusError(BTRC_ERR_CUDA, msg);
            if(gs == GpuBvhStatus::internal)
                throw StatusError(BTRC_ERR_INTERNAL, msg);
            // no_progress / too_deep: the host builder takes the scene
        }
    }
    if(sc->bvh_builder == 0 && !two)
    {
        CWBVH bvh = build_cwbvh(world, pool);
        sc->bvh_nodes = static_cast<int>(bvh.nodes.size());
        sc->bvh_depth = bvh.depth;
        sc->bvh_bytes = bvh.nodes.size() * sizeof(CWNode) + bvh.tris.size() * sizeof(TriRec);
        if(!host_only)
        {
            D.nodes = reinterpret_cast<const F4 *>(dev_upload(sc->allocs, bvh.nodes.data(), bvh.nodes.size()));
            D.tris = reinterpret_cast<const F4 *>(dev_upload(sc->allocs, bvh.tris.data(), bvh.tris.size()));
            D.node_count = static_cast<uint32_t>(bvh.nodes.size());
            D.tri_count = static_cast<uint32_t>(bvh.tris.size());
        }
        if(keep_host)
        {
            sc->host_nodes = std::move(bvh.nodes);
            sc->host_tris = std::move(bvh.tris);
        }
    }
    world.clear();
    world.shrink_to_fit();
    sc->bvh_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb).count();
    if(host_only)
    {
        sc->built = true;
        sc->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return;
    }

    // shading SoA + geometry table + light sampling data
    std::vector<Geometry> geos(H.geometries.size());
    std::vector<bool> is_light_geo(H.geometries.size(), false);
    for(auto &L : H.area_lights)
        is_light_geo[L.geometry] = true;
    size_t total = 0, light_total = 0;
    for(size_t g = 0; g < H.geometries.size(); ++g)
    {
        geos[g].tri_offset = static_cast<uint32_t>(total);
        geos[g].tri_count = static_cast<uint32_t>(H.geometries[g].area.size());
        geos[g].total_area = H.geometries[g].total_area;
        uint32_t lo = 0xffffffffu;
        if(is_light_geo[g])
        {
            lo = static_cast<uint32_t>(light_total);
            light_total += H.geometries[g].area.size();
        }
        std::memcpy(&geos[g].pad, &lo, sizeof(lo));
        total += H.geometries[g].area.size();
    }
    {
        // interleave the per-geometry component arrays into one record per triangle
        std::vector<F4> rec(total * SHADE_F4);
        size_t first = 0;
        for(auto &g : H.geometries)
        {
            F4 *dst = rec.data() + first * SHADE_F4;
            pool.parallel_for(g.shade[0].size(), 1u << 14, [&g, dst](size_t b, size_t e) {
                for(size_t i = b; i < e; ++i)
                    for(int k = 0; k < SHADE_F4; ++k)
                        dst[i * SHADE_F4 + k] = g.shade[k][i];
            });
            first += g.shade[0].size();
        }
        D.shade = dev_upload(sc->allocs, rec.data(), rec.size());
    }
    std::vector<F4> lpos;
    std::vector<AliasEntry8> lalias;
    lpos.reserve(light_total * 3);
    lalias.reserve(light_total);
    for(size_t g = 0; g < H.geometries.size(); ++g)
    {
        if(!is_light_geo[g])
            continue;
        const HostGeometry &G = H.geometries[g];
        for(size_t t = 0; t < G.area.size(); ++t)
        {
            // the w components carry the triangle's geometric normal (shading record 2), so
            // that a light sample reads one 48-byte record
            const V3 a = G.pos[t * 3], ba = G.pos[t * 3 + 1] - a, ca = G.pos[t * 3 + 2] - a;
            const F4 gz = G.shade[2][t];
            lpos.push_back({ a.x, a.y, a.z, gz.x });
            lpos.push_back({ ba.x, ba.y, ba.z, gz.y });
            lpos.push_back({ ca.x, ca.y, ca.z, gz.z });
        }
        auto tab = build_alias_table(G.area);
        lalias.insert(lalias.end(), tab.begin(), tab.end());
    }
    sc->n_shade_tris = total;
    sc->n_light_tris = light_total;
    D.geometries = dev_upload(sc->allocs, geos.data(), geos.size());
    D.instances = dev_upload(sc->allocs, H.instances.data(), H.instances.size());
    D.materials = dev_upload(sc->allocs, H.materials.data(), H.materials.size());
    D.area_lights = dev_upload(sc->allocs, H.area_lights.data(), H.area_lights.size());
    D.light_pos = dev_upload(sc->allocs, lpos.data(), lpos.size());
    D.light_alias = dev_upload(sc->allocs, lalias.data(), lalias.size());
    D.num_area_lights = static_cast<int32_t>(H.area_lights.size());
    D.num_lights = D.num_area_lights + (H.env.type != ENV_NONE ? 1 : 0);
    D.env = H.env;

    // media and density grids
    std::vector<Medium> meds;
    std::vector<float> grids;
    for(auto &m : H.media)
    {
        Medium md = m.dev;
        md.grid_offset = static_cast<int32_t>(grids.size());
        grids.insert(grids.end(), m.grid.begin(), m.grid.end());
        meds.push_back(md);
    }
    std::vector<VolumePrim> vols = H.volumes;
    {
        const int32_t base = static_cast<int32_t>(grids.size());
        if(grids.size() + H.volume_grids.size() > static_cast<size_t>(INT32_MAX))
            throw std::runtime_error("density grids exceed 2^31 floats");
        for(VolumePrim &v : vols)
        {
            if(v.sigma_offset >= 0)
                v.sigma_offset += base;
            if(v.albedo_offset >= 0)
                v.albedo_offset += base;
        }
        grids.insert(grids.end(), H.volume_grids.begin(), H.volume_grids.end());
    }
    D.volumes = vols.empty() ? nullptr : dev_upload(sc->allocs, vols.data(), vols.size());
    D.volume_nodes = H.volume_nodes.empty() ? nullptr
                                             : dev_upload(sc->allocs, H.volume_nodes.data(), H.volume_nodes.size());
    D.num_volumes = static_cast<int32_t>(vols.size());
    D.media = dev_upload(sc->allocs, meds.data(), meds.size());
    // textures and the environment map's importance table
    {
        const TexStore &T = H.textures;
        D.tex_images = T.images.empty() ? nullptr : dev_upload(sc->allocs, T.images.data(), T.images.size());
        D.tex_texels = T.texels.empty() ? nullptr : dev_upload(sc->allocs, T.texels.data(), T.texels.size());
        D.tex_instr = T.instr.empty() ? nullptr : dev_upload(sc->allocs, T.instr.data(), T.instr.size());
        D.material_tex = H.material_tex.empty() ? nullptr
                                                 : dev_upload(sc->allocs, H.material_tex.data(), H.material_tex.size());
        D.env_probs = H.env_probs.empty() ? nullptr : dev_upload(sc->allocs, H.env_probs.data(), H.env_probs.size());
        D.env_alias = H.env_alias.empty() ? nullptr : dev_upload(sc->allocs, H.env_alias.data(), H.env_alias.size());
    }
    D.grids = grids.empty() ? nullptr : dev_upload(sc->allocs, grids.data(), grids.size());
    D.num_media = static_cast<int32_t>(meds.size());
    D.vacuum_medium = H.vacuum_medium;
    D.has_media = 0;
    for(auto &inst : H.instances)
    {
        const int inner = static_cast<int>(inst.media & 0xffffu), outer = static_cast<int>(inst.media >> 16);
        if(H.media[inner].dev.type != MED_VACUUM || H.media[outer].dev.type != MED_VACUUM)
            D.has_media = 1;
    }
    if(!vols.empty())
        D.has_media = 1;
    const V3 ext = H.world_max - H.world_min;
    D.world_diagonal = length(ext);
    D.tri_round = TRI_ROUND_TESTS;
    D.shadow_round = TRI_ROUND_SHADOW;

    // film filter table
    if(H.params.filter == FILTER_GAUSSIAN)
    {
        sc->filter_table_host = build_gaussian_filter_table(H.params.filter_radius, H.params.filter_alpha);
        sc->filter_table = dev_upload(sc->allocs, sc->filter_table_host.data(), sc->filter_table_host.size());
    }
    check_cuda(cudaDeviceSynchronize(), "scene upload");
    static std::atomic<uint64_t> build_serial{ 0 };
    sc->serial = ++build_serial;
    sc->built = true;
    sc->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// path queues, shadow queue, hit records, film and counters for `capacity` states
void alloc_render_buffers(RenderBuffers &B, std::vector<void *> &allocs, uint32_t capacity, size_t pixels)
{
    for(void *p : allocs)
        cudaFree(p);
    allocs.clear();
    if(B.host_counters)
        cudaFreeHost(B.host_counters);
    B = RenderBuffers{};
    auto A = [&](size_t bytes) { return dev_alloc(allocs, bytes); };
    for(int k = 0; k < 2; ++k)
    {
        B.path[k].beta_depth = static_cast<F4 *>(A(sizeof(F4) * capacity));
        B.path[k].rad_pixel = static_cast<F4 *>(A(sizeof(F4) * capacity));
        B.path[k].sampler = static_cast<SamplerState *>(A(sizeof(SamplerState) * capacity));
        B.path[k].ray_o = static_cast<F4 *>(A(sizeof(F4) * capacity));
        B.path[k].ray_d = static_cast<F4 *>(A(sizeof(F4) * capacity));
        B.path[k].bsdf_le = static_cast<F4 *>(A(sizeof(F4) * capacity));
    }
    for(int k = 0; k < 2; ++k)
    {
        B.shadow[k].o = static_cast<F4 *>(A(sizeof(F4) * capacity));
        B.shadow[k].d = static_cast<F4 *>(A(sizeof(F4) * capacity));
        B.shadow[k].beta = static_cast<F4 *>(A(sizeof(F4) * capacity));
        B.shadow[k].sampler = static_cast<SamplerState *>(A(sizeof(SamplerState) * capacity));
    }
    B.hit_flag = static_cast<uint32_t *>(A(sizeof(uint32_t) * capacity));
    B.hit_detail = static_cast<HitDetail *>(A(sizeof(HitDetail) * capacity));
    B.order = static_cast<uint32_t *>(A(sizeof(uint32_t) * capacity));
    B.film = static_cast<float4 *>(A(sizeof(float4) * pixels));
    B.counters = static_cast<Counters *>(A(sizeof(Counters)));
    void *hc = nullptr;
    check_cuda(cudaMallocHost(&hc, sizeof(Counters) * RING_SLOTS), "cudaMallocHost");
    B.host_counters = static_cast<Counters *>(hc);
    B.capacity = capacity;
}

void ensure_render_buffers(btrc_ctx *ctx, uint32_t capacity, size_t pixels)
{
    if(ctx->buf_capacity >= capacity && ctx->film_pixels == pixels)
        return;
    check_cuda(cudaStreamSynchronize(ctx->stream), "stream sync");
    ctx->buf_capacity = 0;
    alloc_render_buffers(ctx->buf, ctx->buf_allocs, capacity, pixels);
    ctx->buf_capacity = capacity;
    ctx->film_pixels = pixels;
}

// g-buffer films, allocated the first time a render asks for them
void ensure_aov_buffers(btrc_ctx *ctx, size_t pixels, bool albedo, bool normal)
{
    RenderBuffers &B = ctx->buf;
    if(albedo && !B.aov_albedo)
        B.aov_albedo = static_cast<float4 *>(dev_alloc(ctx->buf_allocs, sizeof(float4) * pixels));
    if(normal && !B.aov_normal)
        B.aov_normal = static_cast<float4 *>(dev_alloc(ctx->buf_allocs, sizeof(float4) * pixels));
}

// device scratch: 256 bytes of error flags, then `images` images of pixels * 3 floats
float *ctx_scratch_images(btrc_ctx *ctx, size_t pixels, int images)
{
    const size_t need = 256 + static_cast<size_t>(images) * pixels * 3 * sizeof(float);
    if(ctx->scratch_bytes < need)
    {
        check_cuda(cudaStreamSynchronize(ctx->stream), "stream sync");
        if(ctx->scratch)
            cudaFree(ctx->scratch);
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
        check_cuda(cudaMalloc(&ctx->scratch, need), "cudaMalloc");
        check_cuda(cudaMemset(ctx->scratch, 0, 256), "cudaMemset");
        ctx->scratch_bytes = need;
    }
    return reinterpret_cast<float *>(static_cast<char *>(ctx->scratch) + 256);
}

float *ctx_denoise_tmp(btrc_ctx *ctx, size_t pixels)
{
    const size_t need = pixels * 3 * sizeof(float);
    if(ctx->denoise_bytes < need)
    {
        check_cuda(cudaStreamSynchronize(ctx->stream), "stream sync");
        if(ctx->denoise_tmp)
            cudaFree(ctx->denoise_tmp);
        ctx->denoise_tmp = nullptr;
        ctx->denoise_bytes = 0;
        check_cuda(cudaMalloc(&ctx->denoise_tmp, need), "cudaMalloc");
        ctx->denoise_bytes = need;
    }
    return ctx->denoise_tmp;
}

DevRender make_render_params(const btrc_scene *sc, int spp, uint32_t capacity)
{
    const HostScene &H = sc->host;
    DevRender R{};
    R.width = H.params.width;
    R.height = H.params.height;
    R.spp = spp;
    R.min_depth = H.params.min_depth;
    R.max_depth = H.params.max_depth;
    R.rr_threshold = H.params.rr_threshold;
    R.rr_cont_prob = H.params.rr_cont_prob;
    R.sampler = H.params.sampler;
    R.filter = H.params.filter;
    R.filter_radius = H.params.filter_radius;
    R.tile = H.params.tile ? 1 : 0;
    R.capacity = capacity;
    R.total_paths = static_cast<uint64_t>(spp) * H.params.width * H.params.height;
    R.halton = halton_consts(H.params.width, H.params.height);
    R.filter_table = sc->filter_table;
    R.cam_eye = H.camera.eye;
    R.cam_lbc = H.camera.lbc;
    R.cam_fx = H.camera.film_x;
    R.cam_fy = H.camera.film_y;
    R.sample_offset = 0;
    R.grid_pct = 100;
    R.nrc_terminate = -1;
    return R;
}

cudaStream_t pick_stream(btrc_ctx *ctx, void *stream)
{
    return stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
}

void require_built(const btrc_scene *sc)
{
    if(!sc || !sc->built)
        throw StatusError(BTRC_ERR_INVALID_ARG, "scene is not built (call btrc_scene_build)");
    if(sc->ctx->device < 0)
        throw StatusError(BTRC_ERR_INVALID_ARG, "host-only context (device -1) cannot run device work");
}

void require_device(const btrc_ctx *ctx)
{
    if(ctx->device < 0)
        throw StatusError(BTRC_ERR_INVALID_ARG, "host-only context (device -1) cannot run device work");
}

uint32_t *ctx_scratch_err(btrc_ctx *ctx)
{
    if(!ctx->scratch)
    {
        check_cuda(cudaMalloc(&ctx->scratch, 256), "cudaMalloc");
        check_cuda(cudaMemset(ctx->scratch, 0, 256), "cudaMemset");
        ctx->scratch_bytes = 256;
    }
    return static_cast<uint32_t *>(ctx->scratch);
}

} // namespace

extern "C" {

const char *btrc_version(void) { return "btrc_gb300 0.1.0 (sm_103a)"; }

btrc_status btrc_ctx_create(int device, btrc_ctx **out)
{
    if(!out)
        return BTRC_ERR_INVALID_ARG;
    *out = nullptr;
    auto ctx = std::make_unique<btrc_ctx>();
    btrc_status s = guarded(nullptr, [&] {
        ctx->device = device;
        if(device == -1)
            return;  // host-only context: scene loading and BVH building, no device work
        int n = 0;
        check_cuda(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
        if(device < 0 || device >= n)
            throw StatusError(BTRC_ERR_INVALID_ARG, "device index out of range");
        ctx->device = device;
        check_cuda(cudaSetDevice(device), "cudaSetDevice");
        check_cuda(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        check_cuda(upload_primes(), "prime table upload");
    });
    if(s == BTRC_OK)
    {
        if(device >= 0)
            noalloc_context_opened(device);
        *out = ctx.release();
    }
    return s;
}

void btrc_ctx_destroy(btrc_ctx *ctx)
{
    if(!ctx)
        return;
    // scenes still alive are destroyed with their context
    while(!ctx->scenes.empty())
        btrc_scene_destroy(*ctx->scenes.begin());
    if(ctx->device < 0)
    {
        delete ctx;
        return;
    }
    cudaSetDevice(ctx->device);
    if(ctx->stream)
        cudaStreamSynchronize(ctx->stream);
    if(!ctx->nrc_allocs.empty())
        cudaDeviceSynchronize();  // a cache's training paths may still be using the context's scratch
    release_render_graph(ctx->buf);
    for(void *p : ctx->buf_allocs)
        cudaFree(p);
    for(void *p : ctx->nrc_allocs)
        cudaFree(p);
    if(ctx->buf.host_counters)
        cudaFreeHost(ctx->buf.host_counters);
    if(ctx->scratch)
        cudaFree(ctx->scratch);
    if(ctx->denoise_tmp)
        cudaFree(ctx->denoise_tmp);
    if(ctx->stream)
        cudaStreamDestroy(ctx->stream);
    noalloc_context_closed(ctx->device);
    delete ctx;
}

const char *btrc_last_error(const btrc_ctx *ctx)
{
    return ctx ? ctx->last_error.c_str() : "null context";
}

void btrc_cancel(btrc_ctx *ctx)
{
    if(ctx)
        ctx->cancel.store(true);
}

btrc_status btrc_scene_load_json(btrc_ctx *ctx, const char *path, btrc_scene **out)
{
    if(!ctx || !path || !out)
        return BTRC_ERR_INVALID_ARG;
    *out = nullptr;
    auto sc = std::make_unique<btrc_scene>();
    sc->ctx = ctx;
    const btrc_status s = guarded(ctx, [&] { sc->host = load_scene(path); });
    if(s == BTRC_OK)
    {
        *out = sc.release();
        ctx->scenes.insert(*out);
    }
    return s;
}

btrc_status btrc_scene_build(btrc_scene *scene, const btrc_build_opts *opts)
{
    if(!scene)
        return BTRC_ERR_INVALID_ARG;
    return guarded(scene->ctx, [&] {
        build_scene(scene, opts ? opts->threads : 0, opts ? opts->builder : 0, opts ? opts->two_level : 0);
    });
}

btrc_status btrc_scenes_load_build(btrc_ctx *ctx, const char *const *paths, uint32_t n, const btrc_build_opts *opts,
                                   btrc_scene **out)
{
    if(!ctx || (n > 0 && (!paths || !out)))
        return BTRC_ERR_INVALID_ARG;
    for(uint32_t i = 0; i < n; ++i)
    {
        out[i] = nullptr;
        if(!paths[i])
            return BTRC_ERR_INVALID_ARG;
    }
    std::vector<std::unique_ptr<btrc_scene>> scs(n);
    std::vector<std::exception_ptr> errors(n);
    const btrc_status s = guarded(ctx, [&] {
        int threads = opts ? opts->threads : 0;
        if(threads <= 0)
            threads = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
        // one pool for everything: scene tasks, and inside them the OBJ pieces, the
        // geometry records and the BVH builds, so small and large scenes share the cores
        TaskPool pool(threads);
        PoolScope scope(pool);
        TaskPool::Group g;
        for(uint32_t i = 0; i < n; ++i)
            pool.run(g, [&, i] {
                try
                {
                    auto sc = std::make_unique<btrc_scene>();
                    sc->ctx = ctx;
                    sc->host = load_scene(paths[i]);
                    if(ctx->device >= 0)
                        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
                    build_scene(sc.get(), threads, opts ? opts->builder : 0, opts ? opts->two_level : 0);
                    scs[i] = std::move(sc);
                }
                catch(...)
                {
                    errors[i] = std::current_exception();
                }
            });
        pool.wait(g);
        // the first scene that failed reports, classified like a single load / build
        for(uint32_t i = 0; i < n; ++i)
            if(errors[i])
                std::rethrow_exception(errors[i]);
    });
    if(s != BTRC_OK)
        return s;  // the scenes built so far are freed with scs
    for(uint32_t i = 0; i < n; ++i)
    {
        out[i] = scs[i].release();
        ctx->scenes.insert(out[i]);
    }
    return BTRC_OK;
}

btrc_status btrc_scene_info_get(const btrc_scene *sc, btrc_scene_info *out)
{
    if(!sc || !out)
        return BTRC_ERR_INVALID_ARG;
    const HostScene &H = sc->host;
    btrc_scene_info i{};
    i.width = H.params.width;
    i.height = H.params.height;
    i.spp = H.params.spp;
    i.min_depth = H.params.min_depth;
    i.max_depth = H.params.max_depth;
    i.state_count = H.params.state_count;
    i.sampler = H.params.sampler;
    i.filter = H.params.filter;
    i.instances = static_cast<int32_t>(H.instances.size());
    i.geometries = static_cast<int32_t>(H.geometries.size());
    i.materials = static_cast<int32_t>(H.materials.size());
    i.area_lights = static_cast<int32_t>(H.area_lights.size());
    i.media = static_cast<int32_t>(H.media.size());
    i.has_envir_light = H.env.type != ENV_NONE ? 1 : 0;
    i.triangles = H.triangle_count;
    i.bvh_nodes = sc->bvh_nodes;
    i.bvh_depth = sc->bvh_depth;
    i.bvh_bytes = sc->bvh_bytes;
    i.world_min[0] = H.world_min.x; i.world_min[1] = H.world_min.y; i.world_min[2] = H.world_min.z;
    i.world_max[0] = H.world_max.x; i.world_max[1] = H.world_max.y; i.world_max[2] = H.world_max.z;
    i.build_ms = sc->build_ms;
    i.bvh_ms = sc->bvh_ms;
    i.bvh_builder = sc->bvh_builder;
    i.two_level = sc->two_level ? 1 : 0;
    *out = i;
    return BTRC_OK;
}

void btrc_scene_destroy(btrc_scene *scene)
{
    if(!scene)
        return;
    btrc_ctx *ctx = scene->ctx;
    if(ctx->scenes.erase(scene) == 0)
        return;  // not a live scene of its context (already destroyed with it)
    if(ctx->device >= 0)
    {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        free_all(scene->allocs);
    }
    delete scene;
}

btrc_status btrc_scene_export_triangles(const btrc_scene *sc, float *xyz, uint32_t *ids, uint64_t capacity)
{
    if(!sc)
        return BTRC_ERR_INVALID_ARG;
    if(!sc->built)
        return BTRC_ERR_INVALID_ARG;
    const uint64_t n = sc->export_count;
    if(capacity < n)
        return BTRC_ERR_INVALID_ARG;
    // recomputed on request (tests and tools), so that builds do not keep a second copy
    const HostScene &H = sc->host;
    uint64_t k = 0;
    for(size_t i = 0; i < H.instances.size(); ++i)
    {
        const size_t m = H.geometries[H.instances[i].geometry].area.size();
        for(size_t t = 0; t < m && k < n; ++t, ++k)
        {
            const TriRec r = world_triangle(H, i, t);
            if(xyz)
            {
                const float v[9] = { r.v0x, r.v0y, r.v0z, r.v1x, r.v1y, r.v1z, r.v2x, r.v2y, r.v2z };
                std::memcpy(xyz + k * 9, v, sizeof(v));
            }
            if(ids)
            {
                ids[k * 2] = r.inst;
                ids[k * 2 + 1] = r.prim;
            }
        }
    }
    return BTRC_OK;
}

btrc_status btrc_scene_export_bvh(const btrc_scene *sc, void *nodes, uint64_t node_capacity, void *tris,
                                  uint64_t tri_capacity)
{
    if(!sc || !sc->built)
        return BTRC_ERR_INVALID_ARG;
    if(sc->host_nodes.size() != static_cast<size_t>(sc->bvh_nodes))
        return BTRC_ERR_UNSUPPORTED;
    if(node_capacity < sc->host_nodes.size() || tri_capacity < sc->host_tris.size())
        return BTRC_ERR_INVALID_ARG;
    if(nodes)
        std::memcpy(nodes, sc->host_nodes.data(), sc->host_nodes.size() * sizeof(CWNode));
    if(tris)
        std::memcpy(tris, sc->host_tris.data(), sc->host_tris.size() * sizeof(TriRec));
    return BTRC_OK;
}

btrc_status btrc_render(btrc_ctx *ctx, btrc_scene *scene, const btrc_render_opts *opts, float *rgb_out,
                        btrc_stats *stats)
{
    if(!ctx || !scene || !rgb_out)
        return BTRC_ERR_INVALID_ARG;
    bool cancelled = false;
    const btrc_status s = guarded(ctx, [&] {
        require_built(scene);
        const auto w0 = std::chrono::steady_clock::now();
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        ctx->cancel.store(false);
        const HostScene &H = scene->host;
        const int spp = opts && opts->spp > 0 ? opts->spp : H.params.spp;
        const int sc_count = opts && opts->state_count > 0 ? opts->state_count : H.params.state_count;
        const uint64_t total = static_cast<uint64_t>(spp) * H.params.width * H.params.height;
        const uint32_t capacity = static_cast<uint32_t>(std::min<uint64_t>(static_cast<uint64_t>(sc_count),
                                                                            std::max<uint64_t>(total, 1)));
        const size_t pixels = static_cast<size_t>(H.params.width) * H.params.height;
        ensure_render_buffers(ctx, capacity, pixels);
        check_cuda(cudaMemsetAsync(ctx->buf.film, 0, sizeof(float4) * pixels, ctx->stream), "film clear");
        const bool post_on = opts && opts->post_process;
        const bool want_albedo = (opts && opts->albedo_out) || (post_on && H.params.albedo);
        const bool want_normal = (opts && opts->normal_out) || (post_on && H.params.normal);
        ensure_aov_buffers(ctx, pixels, want_albedo, want_normal);
        DevRender R = make_render_params(scene, spp, capacity);
        if(want_albedo)
        {
            R.aov_albedo = ctx->buf.aov_albedo;
            check_cuda(cudaMemsetAsync(R.aov_albedo, 0, sizeof(float4) * pixels, ctx->stream), "albedo clear");
        }
        if(want_normal)
        {
            R.aov_normal = ctx->buf.aov_normal;
            check_cuda(cudaMemsetAsync(R.aov_normal, 0, sizeof(float4) * pixels, ctx->stream), "normal clear");
        }
        ctx->buf.capacity = capacity;
        RenderStats rs{};
        const bool graphs = !opts || opts->use_graphs != 0;
        const int profile = opts ? opts->profile : 0;
        if(profile < 0 || profile > 2)
            throw StatusError(BTRC_ERR_INVALID_ARG, "profile must be 0, 1 or 2");
        check_cuda(render_wavefront(scene->dev, R, ctx->buf, ctx->stream, &ctx->cancel, graphs, profile, &rs,
                                    &cancelled),
                   "wavefront render");
        const bool on_dev = opts && opts->output_on_device;
        const bool post = opts && opts->post_process;
        float *rgb_dev = rgb_out, *alb_dev = want_albedo ? (opts ? opts->albedo_out : nullptr) : nullptr,
              *nrm_dev = want_normal ? (opts ? opts->normal_out : nullptr) : nullptr;
        if(!on_dev || (want_albedo && !alb_dev) || (want_normal && !nrm_dev))
        {
            float *img = ctx_scratch_images(ctx, pixels, 3);
            if(!on_dev)
                rgb_dev = img;
            if(want_albedo && (!on_dev || !alb_dev))
                alb_dev = img + pixels * 3;
            if(want_normal && (!on_dev || !nrm_dev))
                nrm_dev = img + pixels * 6;
        }
        check_cuda(launch_resolve(ctx->buf.film, rgb_dev, static_cast<uint32_t>(pixels), ctx->stream), "resolve");
        int extra_launches = 1;
        if(want_albedo)
        {
            check_cuda(launch_resolve_aov(ctx->buf.film, ctx->buf.aov_albedo, alb_dev, static_cast<uint32_t>(pixels),
                                          false, ctx->stream),
                       "albedo resolve");
            ++extra_launches;
        }
        if(want_normal)
        {
            check_cuda(launch_resolve_aov(ctx->buf.film, ctx->buf.aov_normal, nrm_dev, static_cast<uint32_t>(pixels),
                                          true, ctx->stream),
                       "normal resolve");
            ++extra_launches;
        }
        // post_processors in scene order (src/cli/main.cpp:79-80)
        if(post && !cancelled)
        {
            std::vector<float> host_img;
            auto download = [&](const float *d) {
                host_img.resize(pixels * 3);
                check_cuda(cudaMemcpyAsync(host_img.data(), d, pixels * 3 * sizeof(float), cudaMemcpyDeviceToHost,
                                           ctx->stream),
                           "post-process download");
                check_cuda(cudaStreamSynchronize(ctx->stream), "post-process sync");
            };
            for(const PostProcess &q : H.post)
            {
                if(q.type == POST_DENOISE)
                {
                    // guided by the albedo / normal AOVs when the renderer produces them, as the
                    // OptiX denoiser is (postprocess/optix_denoiser.cpp:51-98)
                    check_cuda(launch_denoise_atrous(rgb_dev, ctx_denoise_tmp(ctx, pixels), alb_dev, nrm_dev,
                                                     H.params.width, H.params.height, ctx->stream),
                               "denoise");
                    extra_launches += DENOISE_PASSES;
                    continue;
                }
                if(q.type == POST_TONEMAP)
                {
                    check_cuda(launch_tonemap_aces(rgb_dev, static_cast<uint32_t>(pixels), 3, q.exposure, ctx->stream),
                               "tonemap");
                    ++extra_launches;
                    continue;
                }
                const int w = H.params.width, h = H.params.height;
                try
                {
                    if(!q.color.empty())
                    {
                        download(rgb_dev);
                        save_image(q.color, host_img.data(), w, h, 3, q.gamma);
                    }
                    if(!q.albedo.empty() && want_albedo)
                    {
                        download(alb_dev);
                        save_image(q.albedo, host_img.data(), w, h, 3, 1.0f);
                    }
                    if(!q.normal.empty() && want_normal)
                    {
                        download(nrm_dev);
                        save_image(q.normal, host_img.data(), w, h, 3, 1.0f);
                    }
                }
                catch(const UnsupportedFormat &ex)
                {
                    throw StatusError(BTRC_ERR_UNSUPPORTED, ex.what());
                }
                catch(const std::invalid_argument &ex)
                {
                    throw StatusError(BTRC_ERR_INVALID_ARG, ex.what());
                }
                catch(const std::runtime_error &ex)
                {
                    throw StatusError(BTRC_ERR_IO, ex.what());
                }
            }
        }
        if(!on_dev)
        {
            check_cuda(cudaMemcpyAsync(rgb_out, rgb_dev, pixels * 3 * sizeof(float), cudaMemcpyDeviceToHost,
                                       ctx->stream),
                       "image download");
            if(opts && opts->albedo_out)
                check_cuda(cudaMemcpyAsync(opts->albedo_out, alb_dev, pixels * 3 * sizeof(float),
                                           cudaMemcpyDeviceToHost, ctx->stream),
                           "albedo download");
            if(opts && opts->normal_out)
                check_cuda(cudaMemcpyAsync(opts->normal_out, nrm_dev, pixels * 3 * sizeof(float),
                                           cudaMemcpyDeviceToHost, ctx->stream),
                           "normal download");
        }
        check_cuda(cudaStreamSynchronize(ctx->stream), "render sync");
        if(stats)
        {
            stats->paths = rs.paths;
            stats->extension_rays = rs.ext_rays;
            stats->shadow_rays = rs.shadow_rays;
            stats->bounces = rs.iterations;
            stats->traversal_errors = rs.err;
            stats->device_ms = rs.device_ms;
            stats->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
            stats->kernel_launches = rs.kernel_launches + extra_launches;  // + resolves, tonemaps
            for(int k = 0; k < 6; ++k)
            {
                stats->stage_ms[k] = rs.stage_ms[k];
                stats->stage_launches[k] = rs.stage_launches[k];
            }
            stats->node_visits = rs.node_visits;
            stats->tri_tests = rs.tri_tests;
        }
        if(rs.err)
            throw StatusError(BTRC_ERR_INTERNAL, "traversal stack overflow reported by the device");
    });
    if(s == BTRC_OK && cancelled)
    {
        ctx->last_error = "render cancelled";
        return BTRC_ERR_CANCELLED;
    }
    return s;
}

btrc_status btrc_render_noalloc(btrc_ctx *ctx, btrc_scene *scene, int32_t spp, float *d_rgb_out, btrc_stats *stats)
{
    if(!ctx || !scene || !d_rgb_out || spp < 0)
        return BTRC_ERR_INVALID_ARG;
    bool cancelled = false;
    const btrc_status s = guarded(ctx, [&] {
        require_built(scene);
        const HostScene &H = scene->host;
        const uint64_t pixels = static_cast<uint64_t>(H.params.width) * H.params.height;
        if(pixels > noalloc_max_pixels())
            throw StatusError(BTRC_ERR_INVALID_ARG,
                              "btrc_render_noalloc: film of " + std::to_string(pixels) + " pixels exceeds the " +
                                  std::to_string(noalloc_max_pixels()) + "-pixel limit of its fixed scratch");
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        // k_resolve writes width*height*3 floats through d_rgb_out: it must be device (or
        // managed) memory of this context's device, never a host address
        cudaPointerAttributes attr{};
        if(cudaPointerGetAttributes(&attr, d_rgb_out) != cudaSuccess)
        {
            cudaGetLastError();
            throw StatusError(BTRC_ERR_INVALID_ARG, "btrc_render_noalloc: d_rgb_out is not a CUDA pointer");
        }
        if((attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged) ||
           (attr.type == cudaMemoryTypeDevice && attr.device != ctx->device))
            throw StatusError(BTRC_ERR_INVALID_ARG,
                              "btrc_render_noalloc: d_rgb_out must be device memory of device " +
                                  std::to_string(ctx->device));
        void *scratch = nullptr;
        check_cuda(noalloc_scratch_address(ctx->device, &scratch), "cudaGetSymbolAddress(scratch)");
        ctx->cancel.store(false);
        const int n_spp = spp > 0 ? spp : H.params.spp;
        const uint64_t total = static_cast<uint64_t>(n_spp) * pixels;
        const uint32_t capacity = static_cast<uint32_t>(std::min<uint64_t>(
            std::min<uint64_t>(noalloc_max_states(), static_cast<uint64_t>(H.params.state_count)),
            std::max<uint64_t>(total, 1)));
        const DevRender R = make_render_params(scene, n_spp, capacity);
        RenderStats rs{};
        check_cuda(render_wavefront_noalloc(scene->dev, R, scratch, d_rgb_out, ctx->stream, &ctx->cancel, &rs,
                                            &cancelled),
                   "allocation-free render");
        if(stats)
        {
            *stats = btrc_stats{};
            stats->paths = rs.paths;
            stats->extension_rays = rs.ext_rays;
            stats->shadow_rays = rs.shadow_rays;
            stats->bounces = rs.iterations;
            stats->traversal_errors = rs.err;
            stats->kernel_launches = rs.kernel_launches;
            for(int k = 0; k < 6; ++k)
                stats->stage_launches[k] = rs.stage_launches[k];
        }
        if(rs.err)
            throw StatusError(BTRC_ERR_INTERNAL, "traversal stack overflow reported by the device");
    });
    if(s == BTRC_OK && cancelled)
    {
        ctx->last_error = "render cancelled";
        return BTRC_ERR_CANCELLED;
    }
    return s;
}

btrc_status btrc_trace_closest(btrc_ctx *ctx, const btrc_scene *scene, const btrc_ray *d_rays, uint64_t n,
                               uint32_t *d_flags, btrc_hit *d_hits, void *stream)
{
    if(!ctx || !scene || (n > 0 && (!d_rays || !d_flags || !d_hits)) || n > 0xffffffffull)
        return BTRC_ERR_INVALID_ARG;
    return guarded(ctx, [&] {
        require_built(scene);
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        check_cuda(launch_trace_closest(scene->dev, reinterpret_cast<const Ray *>(d_rays), static_cast<uint32_t>(n),
                                        d_flags, reinterpret_cast<HitDetail *>(d_hits), ctx_scratch_err(ctx),
                                        pick_stream(ctx, stream)),
                   "trace_closest launch");
    });
}

btrc_status btrc_trace_any(btrc_ctx *ctx, const btrc_scene *scene, const btrc_ray *d_rays, uint64_t n,
                           uint32_t *d_occluded, void *stream)
{
    if(!ctx || !scene || (n > 0 && (!d_rays || !d_occluded)) || n > 0xffffffffull)
        return BTRC_ERR_INVALID_ARG;
    return guarded(ctx, [&] {
        require_built(scene);
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        check_cuda(launch_trace_any(scene->dev, reinterpret_cast<const Ray *>(d_rays), static_cast<uint32_t>(n),
                                    d_occluded, ctx_scratch_err(ctx), pick_stream(ctx, stream)),
                   "trace_any launch");
    });
}

btrc_status btrc_trace_stats(btrc_ctx *ctx, const btrc_scene *scene, const btrc_ray *d_rays, uint64_t n,
                             uint32_t *d_node_visits, uint32_t *d_tri_tests, void *stream)
{
    if(!ctx || !scene || (n > 0 && (!d_rays || !d_node_visits || !d_tri_tests)) || n > 0xffffffffull)
        return BTRC_ERR_INVALID_ARG;
    return guarded(ctx, [&] {
        require_built(scene);
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        check_cuda(launch_trace_stats(scene->dev, reinterpret_cast<const Ray *>(d_rays), static_cast<uint32_t>(n),
                                      d_node_visits, d_tri_tests, ctx_scratch_err(ctx), pick_stream(ctx, stream)),
                   "trace_stats launch");
    });
}

btrc_status btrc_sampler_batch(btrc_ctx *ctx, int32_t type, int32_t width, int32_t height, const uint32_t *d_pixel_xy,
                               const uint32_t *d_sample_index, uint64_t n, uint32_t dims, float *d_out, void *stream)
{
    if(!ctx || (type != SAMPLER_INDEPENDENT && type != SAMPLER_HALTON) || width <= 0 || height <= 0 ||
       n > 0xffffffffull || (n > 0 && (!d_pixel_xy || !d_sample_index || !d_out)))
        return BTRC_ERR_INVALID_ARG;
    return guarded(ctx, [&] {
        require_device(ctx);
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        check_cuda(launch_sampler_batch(type, width, height, halton_consts(width, height), d_pixel_xy, d_sample_index,
                                        static_cast<uint32_t>(n), dims, d_out, pick_stream(ctx, stream)),
                   "sampler batch");
    });
}

btrc_status btrc_bsdf_batch(btrc_ctx *ctx, int32_t op, const float *d_material, const float *d_wo,
                            const float *d_wi_or_u, uint64_t n, float *d_out, void *stream)
{
    if(!ctx || op < 0 || op > 2 || n > 0xffffffffull || (n > 0 && (!d_material || !d_wo || !d_wi_or_u || !d_out)))
        return BTRC_ERR_INVALID_ARG;
    return guarded(ctx, [&] {
        require_device(ctx);
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        // convert the 16-float records into Material structs on the device
        std::vector<void *> tmp;
        Material *mats = nullptr;
        if(n > 0)
        {
            std::vector<float> hrec(n * 16);
            check_cuda(cudaMemcpy(hrec.data(), d_material, sizeof(float) * n * 16, cudaMemcpyDeviceToHost),
                       "material download");
            std::vector<Material> hm(n);
            for(uint64_t i = 0; i < n; ++i)
            {
                Material m{};
                m.type = static_cast<int32_t>(hrec[i * 16 + 15]);
                if(m.type != MAT_DIFFUSE && m.type != MAT_METAL && m.type != MAT_DISNEY)
                    throw StatusError(BTRC_ERR_INVALID_ARG, "bsdf batch supports diffuse, metal and disney");
                m.shadow_terminator = 0;
                for(int k = 0; k < 15; ++k)
                    m.p[k] = hrec[i * 16 + k];
                hm[i] = m;
            }
            mats = dev_upload(tmp, hm.data(), hm.size());
        }
        cudaError_t e = launch_bsdf_batch(op, mats, d_wo, d_wi_or_u, static_cast<uint32_t>(n), d_out,
                                          pick_stream(ctx, stream));
        if(e == cudaSuccess)
            e = cudaStreamSynchronize(pick_stream(ctx, stream));
        free_all(tmp);
        check_cuda(e, "bsdf batch");
    });
}

btrc_status btrc_medium_tr_batch(btrc_ctx *ctx, const btrc_scene *scene, int32_t medium_id, const float *d_seg,
                                 const uint64_t *d_seeds, uint64_t n, float *d_out, void *stream)
{
    if(!ctx || !scene || n > 0xffffffffull || (n > 0 && (!d_seg || !d_seeds || !d_out)))
        return BTRC_ERR_INVALID_ARG;
    return guarded(ctx, [&] {
        require_built(scene);
        if(medium_id < 0 || medium_id >= scene->dev.num_media)
            throw StatusError(BTRC_ERR_INVALID_ARG, "medium id out of range");
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        check_cuda(launch_medium_tr_batch(scene->dev, medium_id, d_seg, d_seeds, static_cast<uint32_t>(n), d_out,
                                          pick_stream(ctx, stream)),
                   "medium tr batch");
    });
}

btrc_status btrc_tonemap_aces(btrc_ctx *ctx, float *d_pixels, int32_t width, int32_t height, int32_t channels,
                              float exposure, void *stream)
{
    if(!ctx || width < 0 || height < 0 || (channels != 3 && channels != 4) ||
       static_cast<uint64_t>(width) * static_cast<uint64_t>(height) > 0xffffffffull ||
       (width > 0 && height > 0 && !d_pixels))
        return BTRC_ERR_INVALID_ARG;
    return guarded(ctx, [&] {
        if(ctx->device < 0)
            throw StatusError(BTRC_ERR_INVALID_ARG, "host-only context");
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        check_cuda(launch_tonemap_aces(d_pixels, static_cast<uint32_t>(width) * static_cast<uint32_t>(height), channels,
                                       exposure, pick_stream(ctx, stream)),
                   "tonemap");
    });
}

btrc_status btrc_denoise_atrous(btrc_ctx *ctx, float *d_rgb, const float *d_albedo, const float *d_normal,
                                int32_t width, int32_t height, void *stream)
{
    if(!ctx || width < 0 || height < 0 || static_cast<uint64_t>(width) * static_cast<uint64_t>(height) > 0xffffffffull ||
       (width > 0 && height > 0 && !d_rgb))
        return BTRC_ERR_INVALID_ARG;
    return guarded(ctx, [&] {
        if(ctx->device < 0)
            throw StatusError(BTRC_ERR_INVALID_ARG, "host-only context");
        if(width == 0 || height == 0)
            return;
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        cudaStream_t st = pick_stream(ctx, stream);
        float *tmp = ctx_denoise_tmp(ctx, static_cast<size_t>(width) * height);
        check_cuda(launch_denoise_atrous(d_rgb, tmp, d_albedo, d_normal, width, height, st), "denoise");
    });
}

btrc_status btrc_image_load(btrc_ctx *ctx, const char *filename, float *texels, uint64_t capacity, int32_t *width,
                            int32_t *height, int32_t *channels)
{
    if(!filename || !width || !height || !channels)
        return BTRC_ERR_INVALID_ARG;
    return guarded(ctx, [&] {
        LoadedImage img;
        try
        {
            img = load_image(filename);
        }
        catch(const UnsupportedFormat &ex)
        {
            throw StatusError(BTRC_ERR_UNSUPPORTED, ex.what());
        }
        catch(const std::invalid_argument &ex)
        {
            throw StatusError(BTRC_ERR_INVALID_ARG, ex.what());
        }
        catch(const std::runtime_error &ex)
        {
            throw StatusError(BTRC_ERR_IO, ex.what());
        }
        *width = img.width;
        *height = img.height;
        *channels = img.channels;
        if(texels)
        {
            if(capacity < img.texels.size())
                throw StatusError(BTRC_ERR_INVALID_ARG, "texel buffer too small");
            std::memcpy(texels, img.texels.data(), img.texels.size() * sizeof(float));
        }
    });
}

btrc_status btrc_image_save(btrc_ctx *ctx, const char *filename, const float *pixels, int32_t width, int32_t height,
                            int32_t channels, float gamma)
{
    if(!filename || !pixels || width <= 0 || height <= 0 || (channels != 3 && channels != 4) || !(gamma > 0))
        return BTRC_ERR_INVALID_ARG;
    return guarded(ctx, [&] {
        try
        {
            save_image(filename, pixels, width, height, channels, gamma);
        }
        catch(const UnsupportedFormat &ex)
        {
            throw StatusError(BTRC_ERR_UNSUPPORTED, ex.what());
        }
        catch(const std::invalid_argument &ex)
        {
            throw StatusError(BTRC_ERR_INVALID_ARG, ex.what());
        }
        catch(const std::runtime_error &ex)
        {
            throw StatusError(BTRC_ERR_IO, ex.what());
        }
    });
}

// A cache's frame work beside the path tracing: the training paths of a frame run on a
// stream of their own beside its path tracing and fill one of three sample buffers; the
// frame's Adam steps train on them on a second stream beside the next frame's path
// tracing (the weights are read only by inference, which waits for the last Adam steps).
// Whatever else reads or writes the weights or the samples waits first (wait_training).
struct btrc_nrc
{
    btrc_ctx *ctx;
    std::unique_ptr<bt::Nrc> impl;
    cudaStream_t train_stream = nullptr;  // Adam steps
    cudaStream_t path_stream = nullptr;   // training paths
    cudaEvent_t ready = nullptr;          // a point of the frame's own stream to start from
    cudaEvent_t trained = nullptr;        // the last Adam steps done
    cudaEvent_t paths_done[3] = {};       // training paths of each sample buffer traced
    bool pending = false;
    float *samples[3] = {};               // training samples, three frames in rotation
    uint32_t *sample_count = nullptr;     // one counter per buffer
    size_t sample_cap = 0;
    int slot = 0;                         // buffer of the next frame
    float *loss_host = nullptr;           // pinned, one slot per call parity (sum over steps)
    int loss_steps[2] = {};               // Adam steps behind each slot
    int parity = 0;
    void wait_training()
    {
        if(path_stream)
            cudaStreamSynchronize(path_stream);
        if(pending && train_stream)
            cudaStreamSynchronize(train_stream);
        pending = false;
    }
    void free_samples()
    {
        for(float *&p : samples)
        {
            if(p)
                cudaFree(p);
            p = nullptr;
        }
        if(sample_count)
            cudaFree(sample_count);
        sample_count = nullptr;
        sample_cap = 0;
    }
    ~btrc_nrc()
    {
        wait_training();
        free_samples();
        for(cudaEvent_t ev : { ready, trained, paths_done[0], paths_done[1], paths_done[2] })
            if(ev)
                cudaEventDestroy(ev);
        if(train_stream)
            cudaStreamDestroy(train_stream);
        if(path_stream)
            cudaStreamDestroy(path_stream);
        if(loss_host)
            cudaFreeHost(loss_host);
    }
};

namespace {

void ensure_nrc_buffers(btrc_ctx *ctx, size_t pixels)
{
    if(ctx->nrc_pixels >= pixels && ctx->nrc_counts)
        return;
    check_cuda(cudaStreamSynchronize(ctx->stream), "stream sync");
    for(void *p : ctx->nrc_allocs)
        cudaFree(p);
    ctx->nrc_allocs.clear();
    ctx->nrc_pixels = 0;
    auto A = [&](size_t bytes) { return dev_alloc(ctx->nrc_allocs, bytes); };
    ctx->nrc_query = static_cast<float *>(A(sizeof(float) * NRC_QUERY_FLOATS * pixels));
    ctx->nrc_weight = static_cast<float4 *>(A(sizeof(float4) * pixels));
    ctx->nrc_pred = static_cast<float4 *>(A(sizeof(float4) * pixels));
    ctx->nrc_counts = static_cast<uint32_t *>(A(sizeof(uint32_t) * 4));
    for(auto &sp : ctx->nrc_spread)
        sp = static_cast<float2 *>(A(sizeof(float2) * pixels));
    ctx->nrc_pixels = pixels;
}

void ensure_nrc_samples(btrc_nrc *nrc, size_t sample_cap)
{
    if(nrc->sample_cap >= sample_cap && nrc->sample_count)
        return;
    nrc->wait_training();
    nrc->free_samples();
    for(float *&p : nrc->samples)
        check_cuda(cudaMalloc(&p, sizeof(float) * NRC_SAMPLE_FLOATS * std::max<size_t>(sample_cap, 1)),
                   "training samples");
    check_cuda(cudaMalloc(&nrc->sample_count, sizeof(uint32_t) * 3), "training samples");
    check_cuda(cudaMemset(nrc->sample_count, 0, sizeof(uint32_t) * 3), "training samples");
    nrc->sample_cap = sample_cap;
}

} // namespace

btrc_status btrc_render_nrc_frame(btrc_ctx *ctx, btrc_scene *scene, btrc_nrc *nrc, const btrc_nrc_render_opts *opts,
                                  float *rgb_out, btrc_nrc_frame_stats *fstats)
{
    if(!ctx || !scene || !nrc || !opts || !rgb_out)
        return BTRC_ERR_INVALID_ARG;
    bool cancelled = false;
    const btrc_status st = guarded(ctx, [&] {
        require_built(scene);
        const auto w0 = std::chrono::steady_clock::now();
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        if(scene->dev.has_media)
            throw StatusError(BTRC_ERR_UNSUPPORTED, "radiance-cache rendering of scenes with participating media");
        if(opts->train_stride < 0 || opts->train_steps < 0 || opts->train_batch < 0)
            throw StatusError(BTRC_ERR_INVALID_ARG, "negative training option");
        ctx->cancel.store(false);
        const HostScene &H = scene->host;
        const size_t pixels = static_cast<size_t>(H.params.width) * H.params.height;
        const uint32_t capacity = static_cast<uint32_t>(
            std::min<uint64_t>(static_cast<uint64_t>(H.params.state_count), std::max<size_t>(pixels, 1)));
        const size_t sample_cap = static_cast<size_t>(opts->train_steps) * static_cast<size_t>(opts->train_batch);
        ensure_render_buffers(ctx, capacity, pixels);
        ensure_nrc_buffers(ctx, pixels);
        ensure_nrc_samples(nrc, sample_cap);
        if(!nrc->train_stream)
        {
            check_cuda(cudaStreamCreateWithFlags(&nrc->train_stream, cudaStreamNonBlocking), "training stream");
            check_cuda(cudaStreamCreateWithFlags(&nrc->path_stream, cudaStreamNonBlocking), "training stream");
            for(cudaEvent_t *ev : { &nrc->ready, &nrc->trained, &nrc->paths_done[0], &nrc->paths_done[1],
                                    &nrc->paths_done[2] })
                check_cuda(cudaEventCreateWithFlags(ev, cudaEventDisableTiming), "training event");
            check_cuda(cudaMallocHost(&nrc->loss_host, 2 * sizeof(float)), "loss buffer");
            nrc->loss_host[0] = nrc->loss_host[1] = 0.0f;
        }
        cudaStream_t s = ctx->stream;
        const int slot = nrc->slot;
        check_cuda(cudaMemsetAsync(ctx->buf.film, 0, sizeof(float4) * pixels, s), "film clear");
        check_cuda(cudaMemsetAsync(ctx->nrc_counts, 0, sizeof(uint32_t) * 4, s), "counter clear");
        check_cuda(cudaMemsetAsync(nrc->sample_count + slot, 0, sizeof(uint32_t), s), "counter clear");
        DevRender R = make_render_params(scene, 1, capacity);
        R.sample_offset = opts->frame;
        R.nrc_terminate = opts->terminate_vertex;
        R.nrc_spread_c = opts->terminate_vertex >= 0 ? opts->spread_threshold : 0.0f;
        R.nrc_spread[0] = ctx->nrc_spread[0];
        R.nrc_spread[1] = ctx->nrc_spread[1];
        R.nrc_query = ctx->nrc_query;
        R.nrc_weight = ctx->nrc_weight;
        R.nrc_count = ctx->nrc_counts;
        R.nrc_cap = static_cast<uint32_t>(pixels);
        ctx->buf.capacity = capacity;
        const bool on_dev = opts->output_on_device != 0;
        float *rgb_dev = on_dev ? rgb_out : ctx_scratch_images(ctx, pixels, 1);
        uint32_t *err = ctx_scratch_err(ctx);
        // this frame's training paths (they read no weights) on their own stream, beside
        // this frame's path tracing, into this frame's sample buffer. That buffer was last
        // read by the Adam steps of three calls back, which finished before the inference
        // of two calls back, which this stream has passed.
        const bool train_paths = opts->train_stride > 0 && sample_cap > 0;
        if(train_paths)
        {
            cudaStream_t ps = nrc->path_stream;
            check_cuda(cudaEventRecord(nrc->ready, s), "training event");
            check_cuda(cudaStreamWaitEvent(ps, nrc->ready, 0), "training wait");
            const uint32_t stride = static_cast<uint32_t>(opts->train_stride);
            const uint32_t phase = (opts->frame * 7u + 3u) % stride;
            check_cuda(launch_nrc_train_paths(scene->dev, R, stride, phase, opts->frame + (1u << 20), nrc->samples[slot],
                                              nrc->sample_count + slot, static_cast<uint32_t>(sample_cap), err, ps),
                       "training paths");
            check_cuda(cudaEventRecord(nrc->paths_done[slot], ps), "training event");
        }
        RenderStats rs{};
        check_cuda(render_wavefront(scene->dev, R, ctx->buf, s, &ctx->cancel, true, 0, &rs, &cancelled),
                   "wavefront render");
        // the queries and training samples of this frame
        uint32_t counts[4] = {}, ns_frame = 0;
        check_cuda(cudaMemcpyAsync(counts, ctx->nrc_counts, sizeof(counts), cudaMemcpyDeviceToHost, s), "counters");
        if(train_paths)
        {
            check_cuda(cudaStreamWaitEvent(s, nrc->paths_done[slot], 0), "training wait");
            check_cuda(cudaMemcpyAsync(&ns_frame, nrc->sample_count + slot, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                       s),
                       "counters");
        }
        check_cuda(cudaStreamSynchronize(s), "counters");
        const uint32_t nq = std::min<uint32_t>(counts[0], static_cast<uint32_t>(pixels));
        const uint32_t ns = std::min<uint32_t>(ns_frame, static_cast<uint32_t>(sample_cap));
        // inference reads the weights the last Adam steps write
        if(nrc->pending)
            check_cuda(cudaStreamWaitEvent(s, nrc->trained, 0), "training wait");
        if(nq > 0 && opts->terminate_vertex >= 0)
        {
            check_cuda(nrc->impl->infer(ctx->nrc_query, nq, reinterpret_cast<float *>(ctx->nrc_pred), s),
                       "cache inference");
            check_cuda(launch_nrc_splat(ctx->nrc_pred, ctx->nrc_weight, ctx->nrc_counts, static_cast<uint32_t>(pixels),
                                        ctx->buf.film, H.params.width, s),
                       "cache splat");
        }
        check_cuda(launch_resolve(ctx->buf.film, rgb_dev, static_cast<uint32_t>(pixels), s), "resolve");
        // Adam steps on this frame's samples, on the training stream after this frame's
        // inference: the call returns without waiting for them, and the next frame's path
        // tracing runs beside them
        // the last call's loss slot: final once this call's stream work (which waited for
        // those steps) has completed, read after the frame sync below
        const int loss_prev = nrc->parity ^ 1;
        int steps = 0;
        for(int k = 0; k < opts->train_steps; ++k)
            if(static_cast<uint32_t>(k) * static_cast<uint32_t>(opts->train_batch) < ns)
                ++steps;
        if(steps > 0)
        {
            cudaStream_t ts = nrc->train_stream;
            check_cuda(cudaEventRecord(nrc->ready, s), "training event");
            check_cuda(cudaStreamWaitEvent(ts, nrc->ready, 0), "training wait");
            check_cuda(nrc->impl->reset_loss(ts), "cache training");
            for(int k = 0; k < steps; ++k)
            {
                const uint32_t b0 = static_cast<uint32_t>(k) * static_cast<uint32_t>(opts->train_batch);
                const uint32_t nb = std::min<uint32_t>(static_cast<uint32_t>(opts->train_batch), ns - b0);
                check_cuda(
                    nrc->impl->train(nrc->samples[slot] + static_cast<size_t>(b0) * NRC_SAMPLE_FLOATS, nb, true, ts),
                    "cache training");
            }
            check_cuda(nrc->impl->copy_loss_async(nrc->loss_host + nrc->parity, ts), "cache training");
            check_cuda(cudaEventRecord(nrc->trained, ts), "training event");
            nrc->pending = true;
        }
        else
            nrc->loss_host[nrc->parity] = 0.0f;
        nrc->loss_steps[nrc->parity] = steps;
        nrc->parity ^= 1;
        nrc->slot = (slot + 1) % 3;
        if(!on_dev)
            check_cuda(cudaMemcpyAsync(rgb_out, rgb_dev, pixels * 3 * sizeof(float), cudaMemcpyDeviceToHost, s),
                       "image download");
        check_cuda(cudaStreamSynchronize(s), "frame sync");
        check_cuda(nrc->impl->check_error(s), "radiance cache tensor-core kernel");
        if(fstats)
        {
            fstats->paths = rs.paths;
            fstats->queries = nq;
            fstats->train_samples = ns;
            fstats->train_steps = steps;
            // the last frame's training has finished by now (this frame's stream waited for
            // it before inference); this frame's finishes after the call returns
            fstats->loss = nrc->loss_steps[loss_prev] ? nrc->loss_host[loss_prev] / nrc->loss_steps[loss_prev] : 0.0f;
            fstats->render_ms = rs.device_ms;
            fstats->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
        }
        if(rs.err)
            throw StatusError(BTRC_ERR_INTERNAL, "traversal stack overflow reported by the device");
    });
    if(st == BTRC_OK && cancelled)
    {
        ctx->last_error = "render cancelled";
        return BTRC_ERR_CANCELLED;
    }
    return st;
}

btrc_status btrc_nrc_create(btrc_ctx *ctx, const float bbox_min[3], const float bbox_max[3], uint64_t seed,
                            btrc_nrc **out)
{
    if(!ctx || !bbox_min || !bbox_max || !out)
        return BTRC_ERR_INVALID_ARG;
    *out = nullptr;
    return guarded(ctx, [&] {
        if(ctx->device < 0)
            throw StatusError(BTRC_ERR_INVALID_ARG, "host-only context");
        for(int a = 0; a < 3; ++a)
            if(!(bbox_max[a] >= bbox_min[a]))
                throw StatusError(BTRC_ERR_INVALID_ARG, "empty bounding box");
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        auto n = std::make_unique<btrc_nrc>();
        n->ctx = ctx;
        try
        {
            n->impl = std::make_unique<bt::Nrc>(bbox_min, bbox_max, seed);
        }
        catch(const std::runtime_error &e)
        {
            throw StatusError(BTRC_ERR_CUDA, e.what());
        }
        *out = n.release();
    });
}

void btrc_nrc_destroy(btrc_nrc *nrc)
{
    if(!nrc)
        return;
    if(nrc->ctx && nrc->ctx->device >= 0)
        cudaSetDevice(nrc->ctx->device);
    delete nrc;
}

btrc_status btrc_nrc_infer(btrc_ctx *ctx, btrc_nrc *nrc, const float *d_queries, uint64_t n, float *d_out,
                           void *stream)
{
    if(!ctx || !nrc || n > 0xffffffffull || (n > 0 && (!d_queries || !d_out)))
        return BTRC_ERR_INVALID_ARG;
    return guarded(ctx, [&] {
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        nrc->wait_training();
        check_cuda(nrc->impl->infer(d_queries, static_cast<uint32_t>(n), d_out, pick_stream(ctx, stream)),
                   "radiance cache inference");
    });
}

btrc_status btrc_nrc_train(btrc_ctx *ctx, btrc_nrc *nrc, const float *d_samples, uint64_t n, int32_t apply_adam,
                           float *loss_out)
{
    if(!ctx || !nrc || n > 0xffffffffull || (n > 0 && !d_samples))
        return BTRC_ERR_INVALID_ARG;
    return guarded(ctx, [&] {
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        nrc->wait_training();
        check_cuda(nrc->impl->reset_loss(ctx->stream), "radiance cache training");
        check_cuda(nrc->impl->train(d_samples, static_cast<uint32_t>(n), apply_adam != 0, ctx->stream),
                   "radiance cache training");
        float l = 0.0f;
        check_cuda(nrc->impl->read_loss(&l, ctx->stream), "radiance cache training");
        if(loss_out)
            *loss_out = l;
    });
}

btrc_status btrc_nrc_params(btrc_ctx *ctx, btrc_nrc *nrc, int32_t which, float *host, uint64_t count, int32_t set)
{
    if(!ctx || !nrc || !host || which < 0 || which > 3 || (set && which > 1))
        return BTRC_ERR_INVALID_ARG;
    return guarded(ctx, [&] {
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        nrc->wait_training();
        const cudaError_t e = nrc->impl->copy_params(which, host, count, set != 0, ctx->stream);
        if(e == cudaErrorInvalidValue)
            throw StatusError(BTRC_ERR_INVALID_ARG, "parameter count mismatch");
        check_cuda(e, "radiance cache parameters");
    });
}

BatchLane::~BatchLane()
{
    if(stream)
        cudaStreamSynchronize(stream);
    release_render_graph(buf);
    for(void *p : allocs)
        cudaFree(p);
    if(buf.host_counters)
        cudaFreeHost(buf.host_counters);
    if(rgb)
        cudaFree(rgb);
    if(err)
        cudaFree(err);
    if(stream)
        cudaStreamDestroy(stream);
}

namespace {

int ilog2(uint64_t v)
{
    int r = 0;
    while(v > 1)
    {
        v >>= 1;
        ++r;
    }
    return r;
}

std::pair<int, int> scene_class(const btrc_scene *sc)
{
    const uint64_t pixels = static_cast<uint64_t>(sc->host.params.width) * sc->host.params.height;
    return { ilog2(pixels), ilog2(std::max<uint64_t>(sc->host.triangle_count, 1)) / 2 };
}

void lane_prepare(BatchLane &L, uint32_t capacity, size_t pixels, bool host_out)
{
    if(!L.stream)
        check_cuda(cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking), "cudaStreamCreate");
    if(!L.err)
    {
        check_cuda(cudaMalloc(&L.err, 256), "cudaMalloc");
        check_cuda(cudaMemset(L.err, 0, 256), "cudaMemset");
    }
    if(L.capacity < capacity || L.pixels < pixels)
    {
        check_cuda(cudaStreamSynchronize(L.stream), "stream sync");
        const uint32_t cap = std::max(L.capacity, capacity);
        const size_t px = std::max(L.pixels, pixels);
        L.capacity = 0;
        alloc_render_buffers(L.buf, L.allocs, cap, px);
        L.capacity = cap;
        L.pixels = px;
    }
    if(host_out && L.rgb_pixels < pixels)
    {
        check_cuda(cudaStreamSynchronize(L.stream), "stream sync");
        if(L.rgb)
            cudaFree(L.rgb);
        L.rgb = nullptr;
        L.rgb_pixels = 0;
        check_cuda(cudaMalloc(&L.rgb, pixels * 3 * sizeof(float)), "cudaMalloc");
        L.rgb_pixels = pixels;
    }
}

// one scene through one lane; returns the wall milliseconds
double lane_render(btrc_ctx *ctx, BatchLane &L, btrc_scene *sc, uint32_t capacity, int grid_pct, float *out,
                   bool on_dev, int spp_override, RenderStats &rs)
{
    const auto t0 = std::chrono::steady_clock::now();
    const HostScene &H = sc->host;
    const size_t pixels = static_cast<size_t>(H.params.width) * H.params.height;
    const int spp = spp_override > 0 ? spp_override : H.params.spp;
    const uint64_t total = static_cast<uint64_t>(spp) * pixels;
    capacity = static_cast<uint32_t>(std::min<uint64_t>(capacity, std::max<uint64_t>(total, 1)));
    lane_prepare(L, capacity, pixels, !on_dev);
    check_cuda(cudaMemsetAsync(L.buf.film, 0, sizeof(float4) * pixels, L.stream), "film clear");
    DevRender R = make_render_params(sc, spp, capacity);
    R.grid_pct = grid_pct;
    L.buf.capacity = capacity;
    bool cancelled = false;
    check_cuda(render_wavefront(sc->dev, R, L.buf, L.stream, &ctx->cancel, true, 0, &rs, &cancelled), "batch render");
    if(out)
    {
        float *dst = on_dev ? out : L.rgb;
        check_cuda(launch_resolve(L.buf.film, dst, static_cast<uint32_t>(pixels), L.stream), "resolve");
        if(!on_dev)
            check_cuda(cudaMemcpyAsync(out, L.rgb, pixels * 3 * sizeof(float), cudaMemcpyDeviceToHost, L.stream),
                       "image download");
    }
    check_cuda(cudaStreamSynchronize(L.stream), "lane sync");
    if(rs.err)
        throw StatusError(BTRC_ERR_INTERNAL, "traversal stack overflow reported by the device");
    if(cancelled)
        throw StatusError(BTRC_ERR_CANCELLED, "render cancelled");
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// Autotuner: per scene class, probe queue capacities and grid sizes on one lane with a
// short render (about 2^20 paths) and keep the fastest per path.
void autotune(btrc_ctx *ctx, btrc_scene *const *scenes, uint32_t n)
{
    if(ctx->lanes.empty())
        ctx->lanes.push_back(std::make_unique<BatchLane>());
    BatchLane &L = *ctx->lanes[0];
    for(uint32_t i = 0; i < n; ++i)
    {
        const auto key = scene_class(scenes[i]);
        if(ctx->tuned.count(key))
            continue;
        const HostScene &H = scenes[i]->host;
        const uint64_t pixels = static_cast<uint64_t>(H.params.width) * H.params.height;
        const int probe_spp = static_cast<int>(std::max<uint64_t>(1, std::min<uint64_t>(H.params.spp, (1u << 20) / pixels)));
        double best = 1e300;
        std::pair<uint32_t, int> choice{ 1u << 20, 100 };
        for(uint32_t cap : { 1u << 18, 1u << 19, 1u << 20, 1u << 21 })
        {
            if(cap > 4 * pixels * probe_spp && cap != (1u << 18))
                continue;
            for(int pct : { 100, 50 })
            {
                RenderStats rs{};
                lane_render(ctx, L, scenes[i], cap, pct, nullptr, true, probe_spp, rs);  // warm
                const double ms = lane_render(ctx, L, scenes[i], cap, pct, nullptr, true, probe_spp, rs);
                const double per_path = ms / static_cast<double>(std::max<uint64_t>(rs.paths, 1));
                if(per_path < best)
                {
                    best = per_path;
                    choice = { cap, pct };
                }
            }
        }
        ctx->tuned[key] = choice;
    }
}

} // namespace

namespace {

// The scenes of a merged batch, concatenated on the device: each scene's arrays are copied
// behind the previous scenes' and the indices its records hold are shifted by the offsets
// of its slices. Scenes without media, textures, image-based lights or volume primitives
// (what the merged stage kernels read per scene: BVH root, lights, sky, camera, film).
std::unique_ptr<MergedBatch> merge_scenes(btrc_ctx *ctx, btrc_scene *const *scenes, uint32_t n)
{
    if(n == 0 || n > 255)
        throw StatusError(BTRC_ERR_INVALID_ARG, "a merged batch holds 1 to 255 scenes");
    auto mb = std::make_unique<MergedBatch>();
    uint64_t nodes = 0, tris = 0, inst = 0, geos = 0, mats = 0, lights = 0, meds = 0, shade = 0, ltris = 0, rows = 0;
    uint32_t width = 0;
    for(uint32_t i = 0; i < n; ++i)
    {
        const btrc_scene *sc = scenes[i];
        const DevScene &D = sc->dev;
        const HostScene &H = sc->host;
        if(D.has_media || D.material_tex || D.num_volumes || D.env.type == ENV_IBL)
            throw StatusError(BTRC_ERR_UNSUPPORTED,
                              "merged batches take scenes without media, textures, image lights or volumes");
        if(D.node_count == 0)
            throw StatusError(BTRC_ERR_UNSUPPORTED, "merged batches take scenes with at least one triangle");
        if(D.two_level)
            throw StatusError(BTRC_ERR_UNSUPPORTED, "merged batches take single-level scenes");
        if(H.params.width > 65535)
            throw StatusError(BTRC_ERR_UNSUPPORTED, "film too wide for a merged batch");
        nodes += D.node_count;
        tris += D.tri_count;
        inst += H.instances.size();
        geos += H.geometries.size();
        mats += H.materials.size();
        lights += static_cast<uint64_t>(D.num_area_lights);
        meds += static_cast<uint64_t>(D.num_media);
        shade += sc->n_shade_tris;
        ltris += sc->n_light_tris;
        rows += static_cast<uint64_t>(H.params.height);
        width = std::max<uint32_t>(width, static_cast<uint32_t>(H.params.width));
        mb->scenes.push_back(sc);
        mb->serials.push_back(sc->serial);
    }
    if(rows > 65535)
        throw StatusError(BTRC_ERR_UNSUPPORTED, "merged films taller than 65535 rows");
    if(tris >= (1ull << 27) || nodes >= 0xffffffffull)
        throw StatusError(BTRC_ERR_UNSUPPORTED, "merged batch exceeds 2^27 triangle records");
    auto alloc = [&](size_t bytes) { return dev_alloc(mb->allocs, std::max<size_t>(bytes, 16)); };
    CWNode *d_nodes = static_cast<CWNode *>(alloc(nodes * sizeof(CWNode)));
    TriRec *d_tris = static_cast<TriRec *>(alloc(tris * sizeof(TriRec)));
    Instance *d_inst = static_cast<Instance *>(alloc(inst * sizeof(Instance)));
    Geometry *d_geo = static_cast<Geometry *>(alloc(geos * sizeof(Geometry)));
    Material *d_mat = static_cast<Material *>(alloc(mats * sizeof(Material)));
    AreaLight *d_light = static_cast<AreaLight *>(alloc(lights * sizeof(AreaLight)));
    Medium *d_med = static_cast<Medium *>(alloc(meds * sizeof(Medium)));
    F4 *d_shade = static_cast<F4 *>(alloc(shade * SHADE_F4 * sizeof(F4)));
    F4 *d_lpos = static_cast<F4 *>(alloc(ltris * 3 * sizeof(F4)));
    AliasEntry8 *d_lalias = static_cast<AliasEntry8 *>(alloc(ltris * sizeof(AliasEntry8)));
    cudaStream_t st = ctx->stream;
    RebaseOffsets o{};
    uint64_t path_begin = 0;
    uint32_t row_base = 0;
    auto copy = [&](void *dst, const void *src, size_t bytes) {
        if(bytes)
            check_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st), "merged batch copy");
    };
    // queue order: scenes with fewer camera paths first, so that small scenes finish early
    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    auto paths_of = [&](uint32_t i) {
        const HostScene &H = scenes[i]->host;
        return static_cast<uint64_t>(H.params.width) * H.params.height * H.params.spp;
    };
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return paths_of(a) < paths_of(b); });
    mb->input = order;
    for(uint32_t i : order)
    {
        const btrc_scene *sc = scenes[i];
        const DevScene &D = sc->dev;
        const HostScene &H = sc->host;
        const uint32_t n_inst = static_cast<uint32_t>(H.instances.size());
        const uint32_t n_geo = static_cast<uint32_t>(H.geometries.size());
        const uint32_t n_mat = static_cast<uint32_t>(H.materials.size());
        copy(d_nodes + o.node, D.nodes, D.node_count * sizeof(CWNode));
        copy(d_tris + o.tri, D.tris, D.tri_count * sizeof(TriRec));
        copy(d_inst + o.inst, D.instances, n_inst * sizeof(Instance));
        copy(d_geo + o.geo, D.geometries, n_geo * sizeof(Geometry));
        copy(d_mat + o.mat, D.materials, n_mat * sizeof(Material));
        copy(d_light + o.light, D.area_lights, static_cast<size_t>(D.num_area_lights) * sizeof(AreaLight));
        copy(d_med + o.med, D.media, static_cast<size_t>(D.num_media) * sizeof(Medium));
        copy(d_shade + static_cast<size_t>(o.shade_tri) * SHADE_F4, D.shade, sc->n_shade_tris * SHADE_F4 * sizeof(F4));
        copy(d_lpos + static_cast<size_t>(o.light_tri) * 3, D.light_pos, sc->n_light_tris * 3 * sizeof(F4));
        copy(d_lalias + o.light_tri, D.light_alias, sc->n_light_tris * sizeof(AliasEntry8));
        check_cuda(launch_rebase_scene(d_nodes + o.node, D.node_count, d_tris + o.tri, D.tri_count, d_inst + o.inst,
                                       n_inst, d_geo + o.geo, n_geo, d_light + o.light,
                                       static_cast<uint32_t>(D.num_area_lights), o, st),
                   "merged batch rebase");
        BatchScene b{};
        b.R = make_render_params(sc, H.params.spp, 0);
        b.path_begin = path_begin;
        b.row_base = row_base;
        b.root = o.node;
        b.light_begin = static_cast<int32_t>(o.light);
        b.num_area_lights = D.num_area_lights;
        b.num_lights = D.num_lights;
        b.vacuum_medium = D.vacuum_medium + static_cast<int32_t>(o.med);
        b.world_diagonal = D.world_diagonal;
        b.env = D.env;
        mb->table.push_back(b);
        mb->min_depth = std::max(mb->min_depth, H.params.min_depth);
        mb->max_depth = std::max(mb->max_depth, H.params.max_depth);
        path_begin += b.R.total_paths;
        row_base += static_cast<uint32_t>(H.params.height);
        o.node += D.node_count;
        o.tri += D.tri_count;
        o.inst += n_inst;
        o.geo += n_geo;
        o.mat += n_mat;
        o.light += static_cast<uint32_t>(D.num_area_lights);
        o.med += static_cast<uint32_t>(D.num_media);
        o.shade_tri += static_cast<uint32_t>(sc->n_shade_tris);
        o.light_tri += static_cast<uint32_t>(sc->n_light_tris);
    }
    std::vector<uint8_t> row_scene(rows);
    for(uint32_t i = 0; i < n; ++i)
        std::fill(row_scene.begin() + mb->table[i].row_base,
                  row_scene.begin() + mb->table[i].row_base + mb->table[i].R.height, static_cast<uint8_t>(i));
    mb->d_table = dev_upload(mb->allocs, mb->table.data(), mb->table.size());
    mb->d_row_scene = dev_upload(mb->allocs, row_scene.data(), row_scene.size());
    mb->d_outs = static_cast<BatchOut *>(alloc(n * sizeof(BatchOut)));
    mb->film_width = width;
    mb->film_rows = static_cast<uint32_t>(rows);
    mb->total_paths = path_begin;
    DevScene &S = mb->S;
    S = scenes[order[0]]->dev;
    S.nodes = reinterpret_cast<const F4 *>(d_nodes);
    S.tris = reinterpret_cast<const F4 *>(d_tris);
    S.node_count = static_cast<uint32_t>(nodes);
    S.tri_count = static_cast<uint32_t>(tris);
    S.shade = d_shade;
    S.geometries = d_geo;
    S.instances = d_inst;
    S.materials = d_mat;
    S.area_lights = d_light;
    S.light_pos = d_lpos;
    S.light_alias = d_lalias;
    S.media = d_med;
    S.num_media = static_cast<int32_t>(meds);
    S.has_media = 0;
    check_cuda(cudaStreamSynchronize(st), "merged batch build");
    return mb;
}

bool merged_matches(const MergedBatch *mb, btrc_scene *const *scenes, uint32_t n)
{
    if(!mb || mb->scenes.size() != n)
        return false;
    for(uint32_t i = 0; i < n; ++i)
        if(mb->scenes[i] != scenes[i] || mb->serials[i] != scenes[i]->serial)
            return false;
    return true;
}

// one pass over the whole merged batch: every scene's paths in one queue of `capacity`
// states, through the stage kernels' merged variants under the captured bounce graph
double merged_render(btrc_ctx *ctx, MergedBatch &mb, uint32_t capacity, int block, int grid_pct, float *const *outs,
                     bool on_dev, RenderStats &rs, std::vector<double> *scene_done_ms)
{
    const size_t pixels = static_cast<size_t>(mb.film_width) * mb.film_rows;
    capacity = static_cast<uint32_t>(std::min<uint64_t>(capacity, std::max<uint64_t>(mb.total_paths, 1)));
    ensure_render_buffers(ctx, capacity, pixels);
    cudaStream_t st = ctx->stream;
    const auto t0 = std::chrono::steady_clock::now();
    check_cuda(cudaMemsetAsync(ctx->buf.film, 0, sizeof(float4) * pixels, st), "film clear");
    DevRender R{};
    R.width = static_cast<int32_t>(mb.film_width);
    R.height = static_cast<int32_t>(mb.film_rows);
    R.spp = 1;
    R.min_depth = mb.min_depth;
    R.max_depth = mb.max_depth;
    R.sampler = mb.table[0].R.sampler;
    R.capacity = capacity;
    R.total_paths = mb.total_paths;
    R.grid_pct = grid_pct;
    R.nrc_terminate = -1;
    R.batch = mb.d_table;
    R.row_scene = mb.d_row_scene;
    R.batch_count = static_cast<uint32_t>(mb.table.size());
    R.stage_block = block;
    ctx->buf.capacity = capacity;
    bool cancelled = false;
    std::vector<std::pair<double, uint64_t>> progress;
    std::vector<uint8_t> live;
    check_cuda(render_wavefront(mb.S, R, ctx->buf, st, &ctx->cancel, true, 0, &rs, &cancelled,
                                scene_done_ms ? &progress : nullptr, scene_done_ms ? &live : nullptr),
               "merged batch render");
    if(outs)
    {
        // device images: the callers' own, or scratch images copied out afterwards
        const uint32_t n = static_cast<uint32_t>(mb.table.size());
        std::vector<BatchOut> o(n);
        size_t scratch_px = 0;
        uint32_t max_px = 0;
        for(uint32_t i = 0; i < n; ++i)
        {
            const DevRender &r = mb.table[i].R;
            max_px = std::max<uint32_t>(max_px, static_cast<uint32_t>(r.width * r.height));
            scratch_px += static_cast<size_t>(r.width) * r.height;
        }
        float *scratch = on_dev ? nullptr : ctx_scratch_images(ctx, scratch_px, 1);
        size_t at = 0;
        for(uint32_t i = 0; i < n; ++i)
        {
            const DevRender &r = mb.table[i].R;
            o[i].rgb = on_dev ? outs[mb.input[i]] : scratch + at * 3;
            o[i].row_base = mb.table[i].row_base;
            o[i].width = static_cast<uint32_t>(r.width);
            o[i].height = static_cast<uint32_t>(r.height);
            at += static_cast<size_t>(r.width) * r.height;
        }
        check_cuda(cudaMemcpyAsync(mb.d_outs, o.data(), n * sizeof(BatchOut), cudaMemcpyHostToDevice, st),
                   "batch outputs");
        check_cuda(launch_resolve_batch(ctx->buf.film, mb.film_width, mb.d_outs, n, max_px, st), "batch resolve");
        if(!on_dev)
            for(uint32_t i = 0; i < n; ++i)
                check_cuda(cudaMemcpyAsync(outs[mb.input[i]], o[i].rgb,
                                           static_cast<size_t>(o[i].width) * o[i].height * 3 * sizeof(float),
                                           cudaMemcpyDeviceToHost, st),
                           "image download");
    }
    check_cuda(cudaStreamSynchronize(st), "merged batch sync");
    if(rs.err)
        throw StatusError(BTRC_ERR_INTERNAL, "traversal stack overflow reported by the device");
    if(cancelled)
        throw StatusError(BTRC_ERR_CANCELLED, "render cancelled");
    if(scene_done_ms)
    {
        // a scene is done after the first launch by which all of its paths were generated
        // and none was left in the queue, plus one launch for the shadow rays of its last
        // vertices (they run beside the next launch)
        const size_t nb = mb.table.size();
        const bool have_live = live.size() == progress.size() * nb;
        const size_t tail = static_cast<size_t>((std::max(mb.max_depth, mb.min_depth) + 3) / 2);
        scene_done_ms->assign(nb, static_cast<double>(rs.device_ms));
        for(size_t i = 0; i < nb; ++i)
        {
            const uint64_t end = mb.table[i].path_begin + mb.table[i].R.total_paths;
            for(size_t k = 0; k < progress.size(); ++k)
            {
                if(progress[k].second < end || (have_live && live[k * nb + i]))
                    continue;
                // without the queue census: as many launches as the longest path can take
                const size_t done = have_live ? k + 1 : k + tail;
                if(done < progress.size())
                    (*scene_done_ms)[i] = progress[done].first;
                break;
            }
        }
    }
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// queue capacity x threads per block of the stage kernels x persistent-grid size: the
// fastest full pass over the batch (each setting timed after a warm-up pass)
void autotune_merged(btrc_ctx *ctx, MergedBatch &mb)
{
    double best = 1e300;
    for(uint32_t cap : { 1u << 21, 1u << 22, 1u << 23, 1u << 24, 1u << 25 })
        for(int block : { 128, 256 })
            for(int pct : { 100, 50 })
            {
                if(pct == 50 && block == 128)
                    continue;
                RenderStats rs{};
                merged_render(ctx, mb, cap, block, pct, nullptr, true, rs, nullptr);
                const double ms = merged_render(ctx, mb, cap, block, pct, nullptr, true, rs, nullptr);
                if(ms < best)
                {
                    best = ms;
                    mb.capacity = cap;
                    mb.block = block;
                    mb.grid_pct = pct;
                }
            }
    mb.tuned = true;
}

} // namespace

btrc_status btrc_render_batch(btrc_ctx *ctx, btrc_scene *const *scenes, uint32_t n, const btrc_batch_opts *opts,
                              float *const *rgb_out, btrc_batch_scene_stats *stats, double *total_ms)
{
    if(!ctx || (n > 0 && (!scenes || !rgb_out)))
        return BTRC_ERR_INVALID_ARG;
    return guarded(ctx, [&] {
        if(ctx->device < 0)
            throw StatusError(BTRC_ERR_INVALID_ARG, "host-only context");
        for(uint32_t i = 0; i < n; ++i)
        {
            if(!scenes[i] || !rgb_out[i] || scenes[i]->ctx != ctx)
                throw StatusError(BTRC_ERR_INVALID_ARG, "null scene or output, or scene of another context");
            require_built(scenes[i]);
        }
        check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
        ctx->cancel.store(false);
        const int lanes = opts && opts->lanes > 0 ? opts->lanes : 4;
        const bool on_dev = opts && opts->output_on_device;
        const bool tune = opts && opts->autotune;
        if(opts && opts->merged)
        {
            if(!merged_matches(ctx->merged.get(), scenes, n))
            {
                check_cuda(cudaStreamSynchronize(ctx->stream), "stream sync");
                ctx->merged.reset();
                ctx->merged = merge_scenes(ctx, scenes, n);
            }
            MergedBatch &mb = *ctx->merged;
            if(tune && !mb.tuned)
                autotune_merged(ctx, mb);
            const uint32_t cap = mb.tuned ? mb.capacity : static_cast<uint32_t>(scenes[0]->host.params.state_count);
            const int block = mb.tuned ? mb.block : 0, pct = mb.tuned ? mb.grid_pct : 100;
            RenderStats rs{};
            std::vector<double> done;
            const double ms = merged_render(ctx, mb, cap, block, pct, rgb_out, on_dev, rs, stats ? &done : nullptr);
            if(total_ms)
                *total_ms = ms;
            if(stats)
                for(uint32_t k = 0; k < n; ++k)
                {
                    btrc_batch_scene_stats &sst = stats[mb.input[k]];
                    sst.paths = mb.table[k].R.total_paths;
                    sst.ms = done[k];
                    sst.done_ms = done[k];
                    sst.lane = 0;
                    sst.capacity = static_cast<uint32_t>(std::min<uint64_t>(cap, mb.total_paths));
                    sst.grid_pct = pct;
                    sst.block = block > 0 ? block : 256;
                }
            return;
        }
        if(tune)
            autotune(ctx, scenes, n);
        while(static_cast<int>(ctx->lanes.size()) < lanes)
            ctx->lanes.push_back(std::make_unique<BatchLane>());
        // longest processing time first onto the least loaded lane
        std::vector<uint32_t> order(n);
        std::iota(order.begin(), order.end(), 0u);
        auto work = [&](uint32_t i) {
            const HostScene &H = scenes[i]->host;
            return static_cast<double>(H.params.width) * H.params.height * H.params.spp;
        };
        std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return work(a) > work(b); });
        std::vector<std::vector<uint32_t>> assign(lanes);
        std::vector<double> load(lanes, 0.0);
        for(uint32_t i : order)
        {
            const int l = static_cast<int>(std::min_element(load.begin(), load.end()) - load.begin());
            assign[l].push_back(i);
            load[l] += work(i);
        }
        std::vector<std::string> errors(lanes);
        std::vector<btrc_status> codes(lanes, BTRC_OK);
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<std::thread> threads;
        for(int l = 0; l < lanes; ++l)
            threads.emplace_back([&, l] {
                try
                {
                    cudaSetDevice(ctx->device);
                    for(uint32_t i : assign[l])
                    {
                        uint32_t cap = static_cast<uint32_t>(scenes[i]->host.params.state_count);
                        int pct = 100;
                        if(tune)
                        {
                            const auto it = ctx->tuned.find(scene_class(scenes[i]));
                            if(it != ctx->tuned.end())
                            {
                                cap = it->second.first;
                                pct = it->second.second;
                            }
                        }
                        RenderStats rs{};
                        const double ms = lane_render(ctx, *ctx->lanes[l], scenes[i], cap, pct, rgb_out[i], on_dev, 0, rs);
                        if(stats)
                        {
                            stats[i].paths = rs.paths;
                            stats[i].ms = ms;
                            stats[i].lane = l;
                            stats[i].capacity = std::min<uint32_t>(
                                cap, static_cast<uint32_t>(std::max<uint64_t>(rs.paths, 1)));
                            stats[i].grid_pct = pct;
                            stats[i].block = 256;
                            stats[i].done_ms =
                                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
                                    .count();
                        }
                    }
                }
                catch(const StatusError &e)
                {
                    codes[l] = e.status;
                    errors[l] = e.what();
                }
                catch(const std::exception &e)
                {
                    codes[l] = BTRC_ERR_INTERNAL;
                    errors[l] = e.what();
                }
            });
        for(auto &t : threads)
            t.join();
        if(total_ms)
            *total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        for(int l = 0; l < lanes; ++l)
            if(codes[l] != BTRC_OK)
                throw StatusError(codes[l], errors[l]);
    });
}

} // extern "C"
