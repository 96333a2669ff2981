// Host-callable launchers for the CUDA kernels (implemented in the .cu files).
#pragma once

#include <atomic>
#include <cstdint>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "device.h"

namespace bt {

// upload the first 1000 primes to constant memory (once per device)
cudaError_t upload_primes();

cudaError_t launch_trace_closest(const DevScene &S, const Ray *rays, uint32_t n, uint32_t *flags,
                                 HitDetail *hits, uint32_t *err, cudaStream_t st);
cudaError_t launch_trace_any(const DevScene &S, const Ray *rays, uint32_t n, uint32_t *occluded,
                             uint32_t *err, cudaStream_t st);
// per-ray node visits and triangle tests of the closest-hit traversal
cudaError_t launch_trace_stats(const DevScene &S, const Ray *rays, uint32_t n, uint32_t *node_visits,
                               uint32_t *tri_tests, uint32_t *err, cudaStream_t st);

struct RenderBuffers
{
    PathSoA path[2];
    ShadowSoA shadow[2];   // by bounce parity
    uint32_t *hit_flag;
    HitDetail *hit_detail;
    uint32_t *order;       // this bounce's queue slots, paths that hit first (trace -> shade)
    float4 *film;          // radiance.rgb, weight per pixel
    float4 *aov_albedo;    // first-hit albedo sums, allocated on demand
    float4 *aov_normal;    // first-hit normal sums, allocated on demand
    Counters *counters;
    Counters *host_counters;  // pinned, ring of RING_SLOTS
    uint32_t capacity;
    struct RenderGraph *graph = nullptr;  // bounce graph, side stream and events kept across renders
};

// Destroys the bounce graph, side stream and events render_wavefront keeps with B.
void release_render_graph(RenderBuffers &B);

constexpr int RING_SLOTS = 4;

enum Stage
{
    STAGE_CONTROL = 0,
    STAGE_GENERATE = 1,
    STAGE_TRACE = 2,
    STAGE_MEDIUM = 3,
    STAGE_SHADE = 4,
    STAGE_SHADOW = 5,
    STAGE_COUNT = 6
};

struct RenderStats
{
    uint64_t paths;
    uint64_t ext_rays;
    uint64_t shadow_rays;
    uint32_t iterations;
    uint32_t err;
    float device_ms;
    uint64_t kernel_launches;
    double stage_ms[STAGE_COUNT];        // profile mode 1: CUDA events around every launch
    uint64_t stage_launches[STAGE_COUNT];
    uint64_t node_visits, tri_tests;     // profile mode 2: traversal counters
};

// Runs the wavefront loop to completion on stream st. The film must be cleared by the
// caller. Returns cudaSuccess or the first CUDA error; *cancelled is set when the cancel
// flag stopped the loop early.
// profile: 0 none (graphs allowed), 1 per-stage CUDA events (no graphs),
//          2 traversal counters in the closest-hit stage (no graphs, slower)
// progress (optional, graphs only): per launch of the two-bounce graph, the milliseconds
// since the loop started at the end of that launch and the camera paths generated by then.
// live (optional, merged batches with progress): per launch, R.batch_count bytes, 1 where
// a path of that scene was still in the queue after the launch
cudaError_t render_wavefront(const DevScene &S, const DevRender &R, RenderBuffers &B, cudaStream_t st,
                             const std::atomic<bool> *cancel, bool use_graphs, int profile, RenderStats *stats,
                             bool *cancelled, std::vector<std::pair<double, uint64_t>> *progress = nullptr,
                             std::vector<uint8_t> *live = nullptr);

// Allocation-free variant of render_wavefront: all scratch (queues, film, counters) lives
// in a fixed device array; see the block comment above render_wavefront_noalloc.
size_t noalloc_scratch_bytes();
uint32_t noalloc_max_states();
uint32_t noalloc_max_pixels();
cudaError_t noalloc_scratch_address(int device, void **out);
void noalloc_context_opened(int device);
void noalloc_context_closed(int device);
cudaError_t render_wavefront_noalloc(const DevScene &S, const DevRender &R, void *scratch, float *rgb_out,
                                     cudaStream_t st, const std::atomic<bool> *cancel, RenderStats *stats,
                                     bool *cancelled);

// radiance / weight -> rgb (3 floats per pixel)
cudaError_t launch_resolve(const float4 *film, float *rgb, uint32_t pixels, cudaStream_t st);

// merged batches of scenes: index shifts applied to one scene's slice of the combined
// arrays (instance light indices stay scene-local), and the per-scene resolve of the
// combined film
struct RebaseOffsets
{
    uint32_t node, tri, inst, geo, mat, light, med, shade_tri, light_tri;
};
cudaError_t launch_rebase_scene(CWNode *nodes, uint32_t n_nodes, TriRec *tris, uint32_t n_tris, Instance *inst,
                                uint32_t n_inst, Geometry *geo, uint32_t n_geo, AreaLight *lights, uint32_t n_lights,
                                const RebaseOffsets &o, cudaStream_t st);
struct BatchOut
{
    float *rgb;               // device image of width * height * 3 floats
    uint32_t row_base, width, height, pad;
};
cudaError_t launch_resolve_batch(const float4 *film, uint32_t film_width, const BatchOut *outs, uint32_t count,
                                 uint32_t max_pixels, cudaStream_t st);
// g-buffer resolve (sum / weight; normals renormalised) into 3 floats per pixel
cudaError_t launch_resolve_aov(const float4 *film, const float4 *aov, float *out, uint32_t pixels, bool normal,
                               cudaStream_t st);
// radiance-cache training paths over the pixels p with p % stride == phase (sample index
// sample_index): emits up to cap training samples (NRC_SAMPLE_FLOATS each)
cudaError_t launch_nrc_train_paths(const DevScene &S, const DevRender &R, uint32_t stride, uint32_t phase,
                                   uint32_t sample_index, float *samples, uint32_t *count, uint32_t cap, uint32_t *err,
                                   cudaStream_t st);
// film += max(pred, 0) * weight.xyz at pixel weight.w, for min(*count, cap) queries
cudaError_t launch_nrc_splat(const float4 *pred, const float4 *weight, const uint32_t *count, uint32_t cap,
                             float4 *film, int width, cudaStream_t st);
// in-place ACES tone map of 3- or 4-channel float pixels
cudaError_t launch_tonemap_aces(float *px, uint32_t pixels, int channels, float exposure, cudaStream_t st);
// denoise post-processor: edge-avoiding a-trous filter, DENOISE_PASSES passes (tap spacing
// 1, 2, 4, 8, 16), in place on 3-float pixels; tmp holds width x height x 3 floats;
// albedo / normal (3 floats per pixel) may be null
constexpr int DENOISE_PASSES = 5;
constexpr float DENOISE_SIGMA_COLOR = 0.5f;   // in c / (1 + c) space, first pass
constexpr float DENOISE_SIGMA_ALBEDO = 0.05f;
constexpr float DENOISE_SIGMA_NORMAL = 0.3f;  // first pass; scaled by the tap spacing
cudaError_t launch_denoise_atrous(float *rgb, float *tmp, const float *albedo, const float *normal, int width,
                                  int height, cudaStream_t st);

// test hooks
cudaError_t launch_sampler_batch(int type, int width, int height, const HaltonConsts &hc,
                                 const uint32_t *pixel_xy, const uint32_t *sample_index, uint32_t n,
                                 uint32_t dims, float *out, cudaStream_t st);
cudaError_t launch_bsdf_batch(int op, const Material *mats, const float *wo, const float *wi_or_u,
                              uint32_t n, float *out, cudaStream_t st);
cudaError_t launch_medium_tr_batch(const DevScene &S, int medium_id, const float *seg, const uint64_t *seeds,
                                   uint32_t n, float *out, cudaStream_t st);

} // namespace bt
