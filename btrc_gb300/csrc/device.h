// Device-resident scene and per-render parameters (plain pointers into HBM).
#pragma once

#include <cstdint>

#include "layout.h"
#include "sampler.cuh"

namespace bt {

constexpr int SHADE_F4 = 6;

struct DevScene
{
    const F4 *nodes;          // CWNode array viewed as float4 (5 per node)
    const F4 *tris;           // TriRec array viewed as float4 (3 per triangle)
    uint32_t node_count;
    uint32_t tri_count;

    // shading records, SHADE_F4 float4 per triangle (AoS: one hit reads 96 contiguous
    // bytes, three 32-byte sectors), concatenated over geometries:
    // (gx, u0) (gy, u1 - u0) (gz, u2 - u0) (n0, v0) (n1 - n0, v1 - v0) (n2 - n0, v2 - v0)
    const F4 *shade;
    const Geometry *geometries;
    const Instance *instances;
    const Material *materials;
    const AreaLight *area_lights;
    const F4 *light_pos;      // a, b-a, c-a per triangle of light geometries (local space); w: geometric normal
    const AliasEntry8 *light_alias;
    int32_t num_area_lights;
    int32_t num_lights;       // area lights + environment (if any)
    EnvLight env;

    const Medium *media;
    const float *grids;
    int32_t num_media;
    int32_t vacuum_medium;
    int32_t has_media;        // any non-vacuum medium referenced by an instance, or volumes[]
    float world_diagonal;
    const VolumePrim *volumes;
    const VolNode *volume_nodes;
    int32_t num_volumes;

    const TexImage *tex_images;
    const float *tex_texels;   // 4 floats per texel
    const TexInstr *tex_instr;
    const MaterialTex *material_tex;
    const float *env_probs;    // ibl tile probabilities
    const AliasEntry8 *env_alias;
    int32_t tri_round;         // pending triangle tests that start a pooled round (closest hit)
    int32_t shadow_round;      // the same for any-hit (shadow) traversal

    // two-level form (two_level != 0): nodes / tris above are the top level over instance
    // boxes (a leaf record holds the instance index in v0.w); every geometry has its own
    // object-space tree in blas_nodes / blas_tris, rooted at blas_root[geometry]
    // (0xffffffff: no triangles)
    const F4 *blas_nodes;
    const F4 *blas_tris;
    const uint32_t *blas_root;
    uint32_t blas_node_count;
    uint32_t blas_tri_count;
    uint32_t instance_count;
    int32_t two_level;
};

// default of DevScene::tri_round: on the 1080p terrain (3.1 M triangles, 32 M-state queue,
// shadow rounds at 24) closest-hit rounds of 16, 20 and 24 pending tests gave 1020.6-1020.9,
// 1027.0 and 1025.7-1025.8 Mpaths/s (two runs each); rounds started for any single test
// traced 5 % slower than 16
constexpr int32_t TRI_ROUND_TESTS = 20;
// default of DevScene::shadow_round: the shadow kernel on the same frame gave 997.8,
// 999.4, 1005.2, 1011.4, 1017.6, 1020.3, 1021.2, 1018.7 and 1011.6 Mpaths/s for rounds of
// 1, 4, 8, 12, 16, 20, 24, 28 and 32 pending tests
constexpr int32_t TRI_ROUND_SHADOW = 24;

struct BatchScene;

struct DevRender
{
    int32_t width, height, spp;
    int32_t min_depth, max_depth;
    float rr_threshold, rr_cont_prob;
    int32_t sampler;
    int32_t filter;
    float filter_radius;
    int32_t tile;
    uint32_t capacity;
    uint64_t total_paths;
    HaltonConsts halton;
    const AliasEntry8 *filter_table;
    V3 cam_eye, cam_lbc, cam_fx, cam_fy;
    float4 *aov_albedo;       // first-hit albedo sums (xyz), or null
    float4 *aov_normal;       // first-hit normal sums (xyz), or null
    uint32_t sample_offset;   // added to every path's sample index (frame-by-frame rendering)
    int32_t grid_pct;         // persistent grids at this percentage of full occupancy (batched lanes)
    // radiance-cache termination: at the first non-delta surface vertex with depth >=
    // nrc_terminate a path writes a cache query and ends (-1: off)
    int32_t nrc_terminate;
    float *nrc_query;         // NRC_QUERY_FLOATS per query
    float4 *nrc_weight;       // path throughput (xyz) and pixel bits (w) per query
    uint32_t *nrc_count;
    uint32_t nrc_cap;
    // path-spread termination (> 0: end a path at its first non-delta vertex whose spread
    // exceeds nrc_spread_c times the primary spread); per queue slot (spread sum / sqrt(a0),
    // sqrt(a0)) in two arrays indexed by bounce parity
    float nrc_spread_c;
    float2 *nrc_spread[2];
    // merged batch of scenes (null for one scene): the stage kernels read each path's
    // scene from the film row of its pixel word, row_scene[y]
    const BatchScene *batch;
    const uint8_t *row_scene;
    uint32_t batch_count;
    int32_t stage_block;      // threads per block of the grid-stride stage kernels (0: BLOCK)
};

// One scene of a merged batch: its own render parameters and the parts of the combined
// scene that are its own. Its geometry, instances, materials and light triangles live in
// the combined arrays (indices rebased); its BVH is a subtree of the combined node array
// reachable only from `root`, and its film is rows [row_base, row_base + height) of the
// combined film.
struct BatchScene
{
    DevRender R;              // camera, film size, spp, depths, sampler, filter; R.total_paths its paths
    uint64_t path_begin;      // global index of its first camera path
    uint32_t row_base;
    uint32_t root;            // root node of its BVH in the combined node array
    int32_t light_begin;      // its first area light in the combined table
    int32_t num_area_lights;
    int32_t num_lights;       // area lights + its environment light
    int32_t vacuum_medium;
    float world_diagonal;
    int32_t pad[3];
    EnvLight env;
};

// Queue counters, resident in device memory for the whole render. Shadow records are
// double-buffered by bounce parity (bounce b appends to queue b & 1), so that the shadow
// kernel of one bounce may run beside the next bounce's kernels.
struct Counters
{
    uint32_t active;       // states in the current queue (survivors + new)
    uint32_t slot_base;    // first slot written by generate this iteration
    uint32_t n_new;        // paths generated this iteration
    uint32_t next_active;  // survivors appended by shade/medium
    uint32_t shadow_n[2];  // shadow records of the last bounce of each parity
    uint32_t err;          // traversal stack overflow flag
    uint32_t iterations;
    uint64_t generated;    // total camera paths generated
    uint64_t gen_base;     // global path index of slot_base
    uint64_t ext_rays;     // extension rays traced
    uint64_t shadow_rays;  // shadow records of bounces whose queue was reused since
    uint64_t node_visits;  // closest-hit node visits (counting mode only)
    uint64_t tri_tests;    // closest-hit triangle tests (counting mode only)
    uint32_t trace_cursor;      // next ray for the warp-refill traversal (reset every bounce)
    uint32_t shadow_cursor[2];  // per shadow queue
    uint32_t hit_count;      // closest-hit results partitioned into the shade order
    uint32_t miss_count;     // (hits from the front, misses from the back)
};

// Structure-of-arrays path state. Two copies (current / next) per render.
struct PathSoA
{
    F4 *beta_depth;    // beta.xyz, depth (int bits)
    F4 *rad_pixel;     // path radiance.xyz, pixel (x | y << 16)
    SamplerState *sampler;
    F4 *ray_o;         // o.xyz, medium id (bits)
    F4 *ray_d;         // d.xyz, t1
    F4 *bsdf_le;       // beta_le.xyz, bsdf pdf (negative: delta)
};

struct ShadowSoA
{
    F4 *o;             // o.xyz, pixel (bits)
    F4 *d;             // d.xyz, t1
    F4 *beta;          // beta_li.xyz, medium id (bits)
    SamplerState *sampler;
};

} // namespace bt
