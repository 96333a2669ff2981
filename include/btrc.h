/*
 * btrc_gb300 C ABI: a GB300-native wavefront path tracer that loads the same scene JSON
 * as AirGuanZ/Btrc and replaces its wavefront renderer, OptiX traversal and stage
 * kernels. Plain pointers and sizes only; no exceptions cross this boundary.
 *
 * Conventions
 *   - Every entry point returns a btrc_status; btrc_last_error(ctx) gives the message.
 *   - The caller owns ray / hit / image buffers; the library owns scene and BVH memory.
 *   - Functions taking `void *stream` enqueue on that cudaStream_t (NULL: the context's
 *     stream) and return without synchronising; all others are synchronous.
 *   - A context is bound to one CUDA device; calls on one context must not overlap.
 *
 * Reference interfaces each entry point replaces (paths inside the Btrc source tree):
 *   btrc_scene_load_json   factory::JSONParser::parse (src/factory/btrc/factory/node/parser.cpp:59-72)
 *                          + factory::create_scene (src/factory/btrc/factory/scene.cpp:5-94)
 *                          + camera/renderer creation in src/cli/main.cpp:45-66
 *   btrc_scene_build       TriangleMesh::commit / Scene::commit acceleration-structure builds
 *                          (src/builtin/btrc/builtin/geometry/triangle_mesh.cpp:24-171,
 *                           src/core/btrc/core/scene.cpp:92-238,
 *                           src/common/btrc/utils/optix/context.cpp:106-215)
 *   btrc_render            WavefrontPathTracer::render (src/builtin/btrc/builtin/renderer/wavefront.cpp:205-325)
 *                          followed by the preview resolve radiance/weight (wavefront/preview.cpp:28-80)
 *   btrc_trace_closest     TracePipeline::trace (src/builtin/btrc/builtin/renderer/wavefront/trace.cpp:118-166)
 *   btrc_trace_any         ShadowPipeline::test occlusion query (wavefront/shadow.cpp:24-76, 140-158)
 *   btrc_cancel            Renderer::stop_async (src/core/btrc/core/renderer.h)
 */
#ifndef BTRC_GB300_H
#define BTRC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum btrc_status
{
    BTRC_OK = 0,
    BTRC_ERR_INVALID_ARG = 1,
    BTRC_ERR_IO = 2,
    BTRC_ERR_PARSE = 3,
    BTRC_ERR_CUDA = 4,
    BTRC_ERR_OOM = 5,
    BTRC_ERR_TIMEOUT = 6,
    BTRC_ERR_CANCELLED = 7,
    BTRC_ERR_UNSUPPORTED = 8,
    BTRC_ERR_INTERNAL = 9
} btrc_status;

typedef struct btrc_ctx btrc_ctx;
typedef struct btrc_scene btrc_scene;

/* 32 bytes: origin + medium id, direction (not necessarily normalised) + t1.
   Hits are accepted for 0 < t <= t1 (reference SoA layout: wavefront/soa.h:8-38). */
typedef struct btrc_ray
{
    float o[3];
    uint32_t medium_id;
    float d[3];
    float t1;
} btrc_ray;

/* 16 bytes: closest-hit detail (reference: trace.cpp:64-78 writes t, prim_id, b1, b2).
   The matching flag word is instance_id | BTRC_HIT_BIT, or 0 on a miss. */
typedef struct btrc_hit
{
    float t;
    uint32_t prim_id;
    float b1;
    float b2;
} btrc_hit;

#define BTRC_HIT_BIT (1u << 30)

typedef struct btrc_scene_info
{
    int32_t width, height, spp;
    int32_t min_depth, max_depth, state_count;
    int32_t sampler;          /* 0 independent (PCG), 1 halton */
    int32_t filter;           /* 0 box, 1 gaussian */
    int32_t instances, geometries, materials, area_lights, media;
    int32_t has_envir_light;
    uint64_t triangles;       /* after instance flattening */
    int32_t bvh_nodes, bvh_depth;
    uint64_t bvh_bytes;       /* nodes + triangle records */
    float world_min[3], world_max[3];
    double build_ms;
    double bvh_ms;            /* the BVH part of build_ms */
    int32_t bvh_builder;      /* the builder that made the BVH: 0 host, 1 device */
    int32_t two_level;        /* 1: two-level form (bvh_* then cover both levels) */
} btrc_scene_info;

typedef struct btrc_build_opts
{
    int32_t threads;          /* host threads for the BVH build; <= 0: all */
    int32_t builder;          /* 0: host binned SAH (default); 1: on the device (PLOC
                                 clustering, then the same 8-wide collapse and layout),
                                 for batches and cold starts; a scene the device build
                                 refuses (non-finite boxes, a tree deeper than the
                                 traversal stack) is built on the host */
    int32_t two_level;        /* 1: one object-space BVH per geometry under a top-level BVH
                                 over the instances (the form of the reference's IAS over
                                 GASes; memory grows with geometries, not instances x
                                 triangles; rays are walked one per thread, so it traces
                                 slower than the flattened form); every level is built
                                 on the host. Not taken by merged batches; host-only
                                 contexts (device < 0) build the flattened form. */
} btrc_build_opts;

typedef struct btrc_render_opts
{
    int32_t spp;              /* 0: use the scene's renderer.spp */
    int32_t state_count;      /* 0: use the scene's renderer.state_count */
    int32_t output_on_device; /* 1: rgb_out is a device pointer, 0: host pointer */
    int32_t use_graphs;       /* 1: capture bounces in CUDA graphs (default behaviour) */
    int32_t profile;          /* 0 off; 1 CUDA events around every stage launch (no graphs);
                                 2 closest-hit traversal counters (no graphs, slower) */
    int32_t post_process;     /* 1: run the scene's post_processors on the result, in order:
                                 tonemap in place, save writes files, denoise runs
                                 btrc_denoise_atrous (guided by the albedo / normal
                                 images when the renderer produces them) */
    float *albedo_out;        /* optional first-hit albedo, width*height*3 floats, same memory
                                 space as rgb_out (wavefront/shade.cpp:133-139, preview.cpp:27-47) */
    float *normal_out;        /* optional first-hit normal (world space, renormalised) */
} btrc_render_opts;

/* stage indices of btrc_stats.stage_ms / stage_launches */
#define BTRC_STAGE_CONTROL 0
#define BTRC_STAGE_GENERATE 1
#define BTRC_STAGE_TRACE 2
#define BTRC_STAGE_MEDIUM 3
#define BTRC_STAGE_SHADE 4
#define BTRC_STAGE_SHADOW 5

typedef struct btrc_stats
{
    uint64_t paths;           /* camera paths completed */
    uint64_t extension_rays;  /* closest-hit rays traced */
    uint64_t shadow_rays;     /* occlusion rays traced */
    uint32_t bounces;         /* wavefront iterations */
    uint32_t traversal_errors;
    double device_ms;         /* GPU time of the wavefront loop (CUDA events) */
    double wall_ms;           /* host wall time of btrc_render, copies included */
    uint64_t kernel_launches; /* kernels launched by the wavefront loop */
    double stage_ms[6];       /* profile 1: summed CUDA-event time per stage */
    uint64_t stage_launches[6];
    uint64_t node_visits;     /* profile 2: closest-hit node visits over the render */
    uint64_t tri_tests;       /* profile 2: closest-hit triangle tests over the render */
} btrc_stats;

const char *btrc_version(void);

/* device >= 0: CUDA device index. device == -1: host-only context that can load scenes
   and build BVHs (btrc_scene_build skips the upload) but runs no device work. */
btrc_status btrc_ctx_create(int device, btrc_ctx **out);
/* Destroys the context and every scene still alive on it; scene handles of a destroyed
   context must not be used again (not even with btrc_scene_destroy). */
void btrc_ctx_destroy(btrc_ctx *ctx);
const char *btrc_last_error(const btrc_ctx *ctx);
/* Ask a running btrc_render on this context to stop between bounces (thread safe). */
void btrc_cancel(btrc_ctx *ctx);

btrc_status btrc_scene_load_json(btrc_ctx *ctx, const char *path, btrc_scene **out);
btrc_status btrc_scene_build(btrc_scene *scene, const btrc_build_opts *opts);
/* Load and build n scenes at once (no counterpart in the reference, which loads one scene
   per process): JSON parsing, OBJ loading, shading records and BVH builds of all scenes
   run as tasks of one pool of opts->threads host threads (<= 0: all cores), so small and
   large scenes share the cores; each scene is uploaded when built. out[i] receives scene
   i. On any failure every scene of the call is released, out[] stays NULL and the first
   failing scene's status and message are returned. */
btrc_status btrc_scenes_load_build(btrc_ctx *ctx, const char *const *paths, uint32_t n, const btrc_build_opts *opts,
                                   btrc_scene **out);
btrc_status btrc_scene_info_get(const btrc_scene *scene, btrc_scene_info *out);
void btrc_scene_destroy(btrc_scene *scene);

/* World-space triangles in flattened (instance, primitive) order: 9 floats each, plus
   the (instance, primitive) pair in ids (2 uint32 each). Either output may be NULL. */
btrc_status btrc_scene_export_triangles(const btrc_scene *scene, float *xyz, uint32_t *ids, uint64_t capacity);

/* Copy of the flattened acceleration structure: 80-byte compressed 8-wide nodes and
   48-byte triangle records (layout in btrc_gb300/csrc/layout.h). Available for host-only
   contexts and scenes of up to 2^20 triangles; BTRC_ERR_UNSUPPORTED otherwise. */
btrc_status btrc_scene_export_bvh(const btrc_scene *scene, void *nodes, uint64_t node_capacity, void *tris,
                                  uint64_t tri_capacity);

/* Render the whole frame: rgb_out receives width*height*3 floats (radiance / weight).
   The albedo / normal g-buffers are produced when opts asks for them, or for the save
   post-processor when the scene's renderer sets "albedo" / "normal" to true. */
btrc_status btrc_render(btrc_ctx *ctx, btrc_scene *scene, const btrc_render_opts *opts, float *rgb_out,
                        btrc_stats *stats);

/* Render the whole frame without allocating any GPU memory during the call (no
   counterpart in the reference). For callers that cannot call cudaMalloc while they run:
   engines that reserve all device memory up front and hand none out later, processes
   under a hard memory budget, and latency-critical threads on which cudaMalloc/cudaFree
   (which synchronise the device) are not allowed. The scene must already be built;
   d_rgb_out is a caller-owned device buffer of width*height*3 floats.
   All scratch (path queues of 32768 states, film, counters) lives in one fixed
   ~15 MB __device__ array that every GPU loading this library reserves until the
   process exits. Limits: width*height <= 262144 (e.g. 512x512), otherwise
   BTRC_ERR_INVALID_ARG. Each call clears the film and counters it needs; calls share the
   array, so calls that overlap on the GPU (other threads, other contexts on the same
   device) race and must be serialised by the caller. The first call on a device looks
   up the array's device address (cudaGetSymbolAddress); make that first call before any
   stream capture. The address is kept while a context is alive on the device and
   dropped with the last one, so do not reset the device (cudaDeviceReset) while a
   context is alive. spp 0 uses the scene's renderer.spp.
   The render runs on the context's own stream, unordered with the caller's streams:
   finish pending work that writes d_rgb_out before the call. d_rgb_out must be device
   (or managed) memory of the context's device, else BTRC_ERR_INVALID_ARG.
   Differences from btrc_render: the scene's post_processors are not run, no albedo /
   normal g-buffers are produced, and at most 32768 paths are in flight whatever the
   scene's renderer.state_count (the image is the same, rendered in more waves). */
btrc_status btrc_render_noalloc(btrc_ctx *ctx, btrc_scene *scene, int32_t spp, float *d_rgb_out, btrc_stats *stats);

/* ACESToneMap::process (src/builtin/btrc/builtin/postprocess/tonemap.cpp:86-101): in place
   on device pixels of 3 (RGB) or 4 (RGBA, alpha untouched) floats:
   c = saturate(x (2.51 x + 0.03) / (x (2.43 x + 0.59) + 0.14)) with x = c * exposure. */
btrc_status btrc_tonemap_aces(btrc_ctx *ctx, float *d_pixels, int32_t width, int32_t height, int32_t channels,
                              float exposure, void *stream);

/* Stand-in for OptixAIDenoiser::process (src/builtin/btrc/builtin/postprocess/optix_denoiser.cpp:51-126),
   whose OptiX AI denoiser is a closed library: an edge-avoiding a-trous wavelet filter
   (Dammertz et al., HPG 2010; 5 passes, tap spacing 1..16) in place on device pixels of 3
   floats, guided by the optional first-hit albedo and normal images (3 floats per pixel,
   NULL = unused). Runs on `stream` (NULL = the context's stream). The `denoise` entry of a
   scene's post_processors runs the same filter. */
btrc_status btrc_denoise_atrous(btrc_ctx *ctx, float *d_rgb, const float *d_albedo, const float *d_normal,
                                int32_t width, int32_t height, void *stream);

/* SaveToImage::process (src/builtin/btrc/builtin/postprocess/save_to_image.cpp:30-61) with
   Image::save (src/common/btrc/utils/image.h:495-550): write host pixels (3 or 4 floats,
   top row first), raised to 1 / gamma, to the format of the file extension: .png (8-bit
   RGBA, byte = min(int(v * 256), 255), alpha 255), .exr (float B, G, R, uncompressed),
   .hdr (RGBE). .jpg / .jpeg: BTRC_ERR_UNSUPPORTED. ctx may be a host-only context; it
   only receives the error message. */
btrc_status btrc_image_save(btrc_ctx *ctx, const char *filename, const float *pixels, int32_t width, int32_t height,
                            int32_t channels, float gamma);

/* ImageDynamic::load (src/common/btrc/utils/image.cpp:296-346) as a 2D texture reads the
   file: .png (1, 3 or 4 channels after palette expansion; 16-bit samples keep their high
   byte) or .hdr (RGBE), as RGBA floats, top row first: 8-bit samples / 255, a one-channel
   image as (v, 0, 0, 1), three channels as (r, g, b, 1). Writes width, height and the
   file's channel count; with texels == NULL only those. capacity is in floats and must
   be at least width*height*4. .jpg / .exr / interlaced PNG: BTRC_ERR_UNSUPPORTED. */
btrc_status btrc_image_load(btrc_ctx *ctx, const char *filename, float *texels, uint64_t capacity, int32_t *width,
                            int32_t *height, int32_t *channels);

/* Closest hit for n device-resident rays. flags[i] = instance | BTRC_HIT_BIT or 0. */
btrc_status btrc_trace_closest(btrc_ctx *ctx, const btrc_scene *scene, const btrc_ray *d_rays, uint64_t n,
                               uint32_t *d_flags, btrc_hit *d_hits, void *stream);

/* Occlusion for n device-resident rays: d_occluded[i] = 1 when any hit in (0, t1]. */
btrc_status btrc_trace_any(btrc_ctx *ctx, const btrc_scene *scene, const btrc_ray *d_rays, uint64_t n,
                           uint32_t *d_occluded, void *stream);

/* Per-ray node visits and triangle tests of the closest-hit traversal (measurement). */
btrc_status btrc_trace_stats(btrc_ctx *ctx, const btrc_scene *scene, const btrc_ray *d_rays, uint64_t n,
                             uint32_t *d_node_visits, uint32_t *d_tri_tests, void *stream);

/* Test hook: sampler streams. For each of n (pixel, sample) pairs write `dims` values
   drawn with get1d from a fresh sampler of the given type (0 independent, 1 halton) for
   a film of width x height. pixel_xy holds x | y << 16. All pointers are device memory. */
btrc_status btrc_sampler_batch(btrc_ctx *ctx, int32_t type, int32_t width, int32_t height,
                               const uint32_t *d_pixel_xy, const uint32_t *d_sample_index, uint64_t n,
                               uint32_t dims, float *d_out, void *stream);

/* Test hook: local-space BSDF component evaluation, device pointers.
   material: 16 floats per record, layout of the scene's material parameters with the
   material type in record[15] (0 diffuse, 1 metal, 2 disney).
   op 0 (eval/pdf): wo, wi: 3 floats each; out: 4 floats (f.rgb, pdf)
   op 1 (sample)  : wo: 3 floats, u: 3 floats; out: 7 floats (f.rgb, pdf, wi.xyz)
   op 2 (direction): as op 1, but only the sampled direction, before Disney's bad-sample
                    rejection; out: 7 floats (1 if a direction was drawn else 0, 0, 0, 0,
                    wi.xyz), for statistical tests of the sampling density against pdf */
btrc_status btrc_bsdf_batch(btrc_ctx *ctx, int32_t op, const float *d_material, const float *d_wo,
                            const float *d_wi_or_u, uint64_t n, float *d_out, void *stream);

/* Test hook: transmittance estimates of medium `medium_id` of a built scene along n
   world-space segments (6 floats: a.xyz, b.xyz); one PCG seed per segment. */
btrc_status btrc_medium_tr_batch(btrc_ctx *ctx, const btrc_scene *scene, int32_t medium_id, const float *d_seg,
                                 const uint64_t *d_seeds, uint64_t n, float *d_out, void *stream);

/* ---- Batched rendering of many scenes (no counterpart in the reference) ------------
   Renders n built scenes (each with its own renderer settings) in one of two ways.
   Lanes: concurrent render lanes, each with its own CUDA stream, path queues and host
   thread, render their share of the scenes with captured per-bounce graphs; scenes go
   longest-first to the least loaded lane. With autotune, each scene class (film size and
   triangle count, in powers of two) gets the queue capacity and persistent-grid size
   that rendered a probe fastest. Merged (opts->merged): the scenes are concatenated into
   one device scene (each scene's BVH, instances, materials and lights become slices of
   combined arrays, its film a band of rows of one film) and every path carries its scene
   in its film row, so one queue and one set of persistent stage kernels render them all;
   autotune picks queue capacity, stage-kernel block size and grid size for the batch.
   Choices are cached in the context; probing happens before the timed batch. */
typedef struct btrc_batch_opts
{
    int32_t lanes;             /* concurrent render lanes (<= 0: 4) */
    int32_t autotune;          /* 1: choose queue capacity and grid size per scene class (lanes), or
                                  queue capacity, stage-kernel block size and grid size (merged) */
    int32_t output_on_device;  /* 1: rgb_out[i] are device pointers, 0: host pointers */
    int32_t merged;            /* 1: one merged pass: every scene's paths in one path queue through
                                  one set of persistent stage kernels under one captured bounce graph
                                  (scenes without media, textures, image lights or volumes; at most
                                  255 scenes, 65535 film rows in total). The concatenated scene is
                                  kept for the next call with the same built scenes. */
} btrc_batch_opts;

typedef struct btrc_batch_scene_stats
{
    uint64_t paths;
    double ms;                 /* lanes: wall time of the scene's render in its lane; merged: as
                                  done_ms */
    int32_t lane;
    uint32_t capacity;         /* queue capacity used */
    int32_t grid_pct;          /* persistent grid size used, percent of full occupancy */
    int32_t block;             /* threads per block of the stage kernels */
    double done_ms;            /* time from the start of the batch's render until the scene's
                                  image was complete. Lanes: wall clock at the end of its render.
                                  Merged: device time to the end of the bounce launch after the
                                  first one that left none of the scene's paths in the queue
                                  (the pass queues scenes with fewer camera paths first) */
} btrc_batch_scene_stats;

/* rgb_out[i]: width_i * height_i * 3 floats for scene i. stats (n entries) and total_ms
   (wall time of the batch, probes excluded) may be NULL. */
btrc_status btrc_render_batch(btrc_ctx *ctx, btrc_scene *const *scenes, uint32_t n, const btrc_batch_opts *opts,
                              float *const *rgb_out, btrc_batch_scene_stats *stats, double *total_ms);

/* ---- Neural radiance cache (no counterpart in the reference) ----------------------
   A multiresolution hash-grid (16 levels x 2 features, 2^19 FP16 entries per level) and
   degree-4 spherical-harmonics encoding of a path vertex feeding a 5 x 64 ReLU MLP with
   BF16 weights and activations and FP32 accumulation, trained online with FP32 Adam
   (lr 1e-2, beta 0.9 / 0.99) on a relative L2 loss. All data pointers are device memory. */
typedef struct btrc_nrc btrc_nrc;

#define BTRC_NRC_QUERY_FLOATS 13   /* position(3), direction to the viewer(3), normal(3), roughness, albedo(3) */
#define BTRC_NRC_SAMPLE_FLOATS 16  /* a query followed by the target radiance (3) */
#define BTRC_NRC_WEIGHTS 22528     /* 80x64 + 4 x 64x64 + 64x16, row-major K x N per layer */
#define BTRC_NRC_HASH_FLOATS 16777216 /* 16 levels x 2^19 entries x 2 features */

/* positions are normalised to [bbox_min, bbox_max]; seed drives the initialisation */
btrc_status btrc_nrc_create(btrc_ctx *ctx, const float bbox_min[3], const float bbox_max[3], uint64_t seed,
                            btrc_nrc **out);
void btrc_nrc_destroy(btrc_nrc *nrc);
/* predicted radiance for n queries: 4 floats per query (rgb, unused) */
btrc_status btrc_nrc_infer(btrc_ctx *ctx, btrc_nrc *nrc, const float *d_queries, uint64_t n, float *d_out,
                           void *stream);
/* one optimisation step over n training samples (apply_adam 0: gradients only, kept until
   the next step); loss_out (host, may be NULL) receives the batch's mean loss */
btrc_status btrc_nrc_train(btrc_ctx *ctx, btrc_nrc *nrc, const float *d_samples, uint64_t n, int32_t apply_adam,
                           float *loss_out);
/* test hook: FP32 host copies of parameters (which 0: MLP weights, 1: hash features) or
   gradients (2: MLP, 3: hash); set != 0 writes parameters 0 / 1 instead */
btrc_status btrc_nrc_params(btrc_ctx *ctx, btrc_nrc *nrc, int32_t which, float *host, uint64_t count, int32_t set);

typedef struct btrc_nrc_render_opts
{
    uint32_t frame;            /* sample index of the frame's single path per pixel */
    int32_t terminate_vertex;  /* paths end in a cache query at the first non-delta surface
                                  vertex of depth >= this (1: after one bounce); -1: no cache */
    int32_t train_stride;      /* one pixel in train_stride traces a training path; 0: none */
    int32_t train_steps;       /* Adam steps per frame */
    int32_t train_batch;       /* training samples per step */
    int32_t output_on_device;  /* 1: rgb_out is a device pointer */
    float spread_threshold;    /* > 0: end paths instead at the first non-delta vertex of depth
                                  >= 1 whose path spread exceeds this times the primary spread
                                  (Mueller et al. 2021, c = 0.01 there); 0: the depth rule */
} btrc_nrc_render_opts;

typedef struct btrc_nrc_frame_stats
{
    uint64_t paths;            /* camera paths of the frame */
    uint64_t queries;          /* paths that ended in a cache query */
    uint64_t train_samples;    /* training samples produced */
    int32_t train_steps;
    float loss;                /* mean training loss of the previous frame's steps (a frame's
                                  Adam steps run on the cache's own stream after the call
                                  returns, beside the next frame's path tracing) */
    double render_ms;          /* GPU time of the wavefront loop */
    double wall_ms;            /* host wall time of the call */
} btrc_nrc_frame_stats;

/* One frame of one path per pixel through the wavefront renderer with paths terminated
   into the radiance cache, training paths for 1 / train_stride of the pixels, cache
   inference and splatting, then the frame's Adam steps. rgb_out receives the frame's
   width*height*3 image (radiance / weight) when the call returns. The training paths
   run on a stream of the cache's own beside the frame's path tracing, and the frame's
   Adam steps on a second such stream that may still be running when the call returns,
   beside the next frame's path tracing. The next frame's inference, btrc_nrc_infer,
   btrc_nrc_train, btrc_nrc_params and btrc_nrc_destroy wait for them. Scenes with
   participating media: BTRC_ERR_UNSUPPORTED. */
btrc_status btrc_render_nrc_frame(btrc_ctx *ctx, btrc_scene *scene, btrc_nrc *nrc, const btrc_nrc_render_opts *opts,
                                  float *rgb_out, btrc_nrc_frame_stats *stats);

#ifdef __cplusplus
}
#endif

#endif /* BTRC_GB300_H */
