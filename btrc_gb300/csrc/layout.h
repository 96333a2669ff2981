// HBM data layout shared by the host builder and the CUDA kernels.
//
// Acceleration structure (single level, instances baked to world space at build time):
//   CWNode  80 B  8-wide compressed node: origin, per-axis power-of-two scale, child
//                 boxes quantised to 8 bits, child/triangle base indices, per-slot meta.
//   TriRec  48 B  world-space triangle v0,v1,v2 (xyz) with the instance index in v0.w
//                 and the primitive index within its geometry in v1.w.
// Shading data (per geometry, shared by all instances of a geometry), 6 x float4 per
// triangle exactly as builtin/btrc/builtin/geometry/triangle_mesh.cpp:40-71 lays it out:
//   ex|u_a, ey|u_ba, ez|u_ca, sn_a|v_a, sn_ba|v_ba, sn_ca|v_ca.
#pragma once

#include <cstdint>

#include "bmath.h"

namespace bt {

struct alignas(16) F4
{
    float x, y, z, w;
};

struct alignas(16) CWNode
{
    float px, py, pz;
    uint8_t ex, ey, ez, imask;
    uint32_t child_base;
    uint32_t tri_base;
    uint8_t meta[8];
    uint8_t qlo_x[8], qlo_y[8], qlo_z[8];
    uint8_t qhi_x[8], qhi_y[8], qhi_z[8];
};
static_assert(sizeof(CWNode) == 80, "CWNode must be 80 bytes");

struct alignas(16) TriRec
{
    float v0x, v0y, v0z;
    uint32_t inst;
    float v1x, v1y, v1z;
    uint32_t prim;
    float v2x, v2y, v2z;
    uint32_t pad;
};
static_assert(sizeof(TriRec) == 48, "TriRec must be 48 bytes");

// Ray as stored in the wavefront queues and passed through btrc_trace_*:
// o.xyz + medium id, d.xyz + t1 (reference: builtin/.../wavefront/soa.h:8-38).
struct alignas(16) Ray
{
    float ox, oy, oz;
    uint32_t medium_id;
    float dx, dy, dz;
    float t1;
};

// Closest-hit result: flag word (instance | HIT_BIT) plus (t, prim, b1, b2).
constexpr uint32_t HIT_BIT = 1u << 30;
constexpr uint32_t SCATTER_BIT = 1u << 29;
constexpr uint32_t INST_MASK = (1u << 29) - 1;

struct alignas(16) HitDetail
{
    float t;
    uint32_t prim;
    float b1, b2;
};

enum MaterialType : int32_t
{
    MAT_DIFFUSE = 0,
    MAT_METAL = 1,
    MAT_DISNEY = 2,
    MAT_BLACK = 3,
    MAT_INVISIBLE = 4,
    MAT_MIRROR = 5,
    MAT_GLASS = 6,
};

// ---- 2D textures (core/btrc/core/texture2d.h, builtin/btrc/builtin/texture2d/*)
// An image texture: RGBA float texels (8-bit files already divided by 255 and, with
// srgb_to_linear, decoded), sampled in normalised coordinates like a CUDA texture object.
enum TexAddress : int32_t
{
    TEX_WRAP = 0,
    TEX_CLAMP = 1,
    TEX_MIRROR = 2,
    TEX_BORDER = 3,
};

struct alignas(16) TexImage
{
    int32_t offset;          // first texel (float4 index) in the texel pool
    int32_t width, height;
    int32_t filter;          // 0 point, 1 linear
    int32_t address_u, address_v;
    int32_t pad[2];
    float border[4];
};

// One instruction of a texture program (postfix): constants and image samples push an RGB
// value, the binary operators of texture2d/math.cpp pop two and push one. uv transforms
// (texture2d/transform.cpp) are folded into the sample instruction's affine map.
enum TexOp : int32_t
{
    TEXOP_END = 0,
    TEXOP_CONST = 1,
    TEXOP_SAMPLE = 2,
    TEXOP_ADD = 3,
    TEXOP_SUB = 4,
    TEXOP_MUL = 5,
    TEXOP_DIV = 6,
};

struct alignas(16) TexInstr
{
    int32_t op;
    int32_t image;           // TEXOP_SAMPLE: index into the image table
    float a[6];              // CONST: rgb in a[0..2]; SAMPLE: u' = a0 u + a1 v + a2, v' = a3 u + a4 v + a5
};

constexpr int TEX_STACK = 8;

// Textured parameters of one material: prog[k] is the first instruction of the program
// that replaces p[k] (k = 0 covers the colour p[0..2]), -1 where p[k] is a constant;
// normal is the normal map's program (material/utils/normal_map.cpp), or -1.
struct alignas(16) MaterialTex
{
    int32_t prog[16];
    int32_t normal;
    int32_t pad[3];
};

// Material parameters (constants, or the values of the textures in MaterialTex).
//   diffuse: p[0..2] albedo
//   metal  : p[0..2] R0, p[3] roughness, p[4] anisotropic
//   disney : p[0..2] base color, p[3] metallic, p[4] roughness, p[5] specular,
//            p[6] specular_tint, p[7] anisotropic, p[8] sheen, p[9] sheen_tint,
//            p[10] clearcoat, p[11] clearcoat_gloss, p[12] transmission,
//            p[13] transmission_roughness, p[14] ior
//   mirror : p[0..2] color
//   glass  : p[0..2] color, p[3] ior
struct alignas(16) Material
{
    int32_t type;
    int32_t shadow_terminator;
    float p[16];
    int32_t tex;             // row of the MaterialTex table, -1: all parameters constant
    int32_t pad;
};

struct alignas(16) Instance
{
    float l2w[12];
    float w2l[12];
    int32_t geometry;
    int32_t material;
    int32_t light;
    uint32_t media;  // inner medium id (low 16) | outer medium id (high 16)
};

struct alignas(16) Geometry
{
    uint32_t tri_offset;  // into the shading SoA and light-sampling arrays
    uint32_t tri_count;
    float total_area;
    float pad;
};

struct alignas(8) AliasEntry8
{
    float accept;
    uint32_t alias;
};

struct alignas(16) AreaLight
{
    int32_t instance;
    int32_t geometry;
    float scale;
    float pad;
    float intensity[3];
    float pad2;
};

enum EnvType : int32_t
{
    ENV_NONE = 0,
    ENV_GRADIENT_SKY = 1,
    ENV_IBL = 2,
};

// Environment light: gradient_sky (builtin/btrc/builtin/light/gradient_sky.cpp) or ibl
// (builtin/btrc/builtin/light/ibl.cpp + env_sampler.cpp): a texture program over the
// (phi / 2 pi, theta / pi) parameterisation of the local frame (frame_x/y/up = from_z(up))
// and a lut_w x lut_h table of tile probabilities with its alias table.
struct alignas(16) EnvLight
{
    int32_t type;
    float lower[3];
    float upper[3];
    float up[3];
    float frame_x[3];
    float frame_y[3];
    int32_t prog;            // ibl texture program
    int32_t lut_w, lut_h;
    int32_t pad;
};

enum MediumType : int32_t
{
    MED_VACUUM = 0,
    MED_HOMOGENEOUS = 1,
    MED_HETEROGENEOUS = 2,
    MED_VOLUMES = 3,      // the volume-primitive medium when the scene has volumes[]
};

// Participating medium. Heterogeneous media are a density grid behind a transform
// (reference: builtin/btrc/builtin/medium/hetergeneous.cpp, core/btrc/core/medium.cpp:98-129).
struct alignas(16) Medium
{
    int32_t type;
    int32_t priority;
    int32_t grid_offset;     // float index into the density pool
    int32_t res_x, res_y, res_z;
    float sigma_max;
    float g;
    float sigma_t_const;     // homogeneous sigma_t (grey) or scale when constant
    float albedo[3];
    float w2l[12];           // world -> medium local ([-1,1]^3) transform
    float l2w[12];
};

// Volume primitive (core/btrc/core/volume.h:9-49): the parallelepiped o + [0,1]^3 (x y z)
// with a sigma_t and an albedo 3D texture over its uvw. Stored in volume-BVH leaf order;
// `id` is its position in the scene's volumes[] array.
struct alignas(16) VolumePrim
{
    float o[3];
    int32_t id;
    float x[3];
    float x_inv_len2;        // world_pos_to_uvw: dot(p - o, x) * (1 / |x|^2) (volume.cpp:45-52)
    float y[3];
    float y_inv_len2;
    float z[3];
    float z_inv_len2;
    float xd[3];             // x / |x|^2: containment and slab tests (volume/bvh.cpp:77-84)
    float sigma_const;       // sigma_t when sigma_offset < 0
    float yd[3];
    float sigma_max;         // Texture3D::get_max_float of sigma_t
    float zd[3];
    int32_t sigma_offset;    // float index of the sigma_t grid in the grid pool, -1: constant
    int32_t sres[3];
    int32_t albedo_offset;   // float index of the albedo grid (3 floats per texel), -1: constant
    int32_t ares[3];
    int32_t albedo_channels; // texels of a 1-channel albedo array read as (v, 0, 0)
    float albedo_const[3];
    float pad;
};

// Binary BVH node over volume boxes: a leaf holds prims [prim_beg, prim_end), an
// interior node has prim_beg = -1 and its children at prim_end and prim_end + 1.
struct alignas(16) VolNode
{
    float lower[3];
    int32_t prim_beg;
    float upper[3];
    int32_t prim_end;
};

constexpr int VOL_MAX_OVERLAP = 4;   // volume/bvh.h:10
constexpr int VOL_STACK = 64;

enum SamplerType : int32_t
{
    SAMPLER_INDEPENDENT = 0,
    SAMPLER_HALTON = 1,
};

// Gaussian filter importance-sampling grid resolution (film_filter/gaussian.cpp:8)
constexpr int FILTER_GRID = 256;

enum FilterType : int32_t
{
    FILTER_BOX = 0,
    FILTER_GAUSSIAN = 1,
};

} // namespace bt
