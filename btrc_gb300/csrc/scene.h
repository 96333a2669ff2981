// Host-side scene model built from a reference-schema scene JSON.
// Mirrors factory/btrc/factory/scene.cpp:5-94 (entities, volumes, envir_light),
// src/cli/main.cpp:45-66 (width/height/camera/renderer) and the builtin creators
// registered in builtin/btrc/builtin/register.cpp:31-113.
#pragma once

#include <string>
#include <vector>

#include "json.h"
#include "layout.h"
#include "textures.h"

namespace bt {

// 4x4 matrix with the reference's Mat4 semantics (common/btrc/utils/math/mat4.cpp):
// at(r, c) is row r, column c.
struct Mat4
{
    float a[4][4];
    static Mat4 identity();
    static Mat4 rows(float m00, float m01, float m02, float m03,
                     float m10, float m11, float m12, float m13,
                     float m20, float m21, float m22, float m23,
                     float m30, float m31, float m32, float m33);
    static Mat4 translate(float x, float y, float z);
    static Mat4 scale(float x, float y, float z);
    static Mat4 rotate(V3 axis, float rad);
    static Mat4 rotate_x(float rad);
    static Mat4 rotate_y(float rad);
    static Mat4 rotate_z(float rad);
};
Mat4 operator*(const Mat4 &a, const Mat4 &b);

// (mat, inv) pair composed like common/btrc/utils/math/transform.cpp:91-124.
struct Transform
{
    Mat4 mat = Mat4::identity();
    Mat4 inv = Mat4::identity();
    V3 point(V3 p) const;
    V3 vector(V3 v) const;
    V3 normal(V3 n) const;
    void to_affine(float l2w[12], float w2l[12]) const;
};
Transform operator*(const Transform &a, const Transform &b);
Transform parse_transform(const json::NodeP &n);

struct HostGeometry
{
    std::string filename;
    std::vector<V3> pos;          // 3 per triangle, object space
    std::vector<F4> shade[6];     // per triangle
    std::vector<float> area;      // per triangle
    float total_area = 0;
    V3 bmin, bmax;
};

struct Camera
{
    V3 eye, lbc, film_x, film_y;
};

struct RenderParams
{
    int width = 0, height = 0;
    int spp = 128;
    int min_depth = 5, max_depth = 10;
    float rr_threshold = 0.1f, rr_cont_prob = 0.5f;
    int state_count = 1000000;
    bool tile = false;
    bool albedo = false, normal = false;
    int filter = FILTER_BOX;
    float filter_radius = 1.3f, filter_alpha = 1.6f;
    int sampler = SAMPLER_INDEPENDENT;
    std::string renderer_type = "wfpt";
};

// Post-processor of the scene's post_processors list (factory/btrc/factory/post_processor.cpp:5-25)
enum PostType : int32_t
{
    POST_SAVE = 0,      // builtin/btrc/builtin/postprocess/save_to_image.cpp:63-76
    POST_TONEMAP = 1,   // builtin/btrc/builtin/postprocess/tonemap.cpp:103-108
    POST_DENOISE = 2,   // optix_denoiser.cpp: run as the a-trous filter (the OptiX denoiser is closed)
};

struct PostProcess
{
    PostType type = POST_SAVE;
    float exposure = 1.0f;    // tonemap
    float gamma = 1.0f;       // save
    std::string color, albedo, normal;  // save: output files ("" = not written)
};

struct HostMedium
{
    Medium dev{};
    float priority = 0;       // sort key of the medium table (descending)
    std::vector<float> grid;  // heterogeneous density (x fastest)
};

struct HostScene
{
    std::string path;
    std::vector<HostGeometry> geometries;
    std::vector<Instance> instances;
    std::vector<Transform> instance_xf;
    std::vector<Material> materials;
    std::vector<MaterialTex> material_tex;  // rows referenced by Material::tex
    TexStore textures;                       // images, texels and texture programs
    std::vector<float> env_probs;            // ibl tile probabilities (lut_w * lut_h)
    std::vector<AliasEntry8> env_alias;
    std::vector<AreaLight> area_lights;
    EnvLight env{};
    std::vector<HostMedium> media;   // index 0 .. n-1; vacuum (volume-primitive medium) included
    int vacuum_medium = 0;
    std::vector<VolumePrim> volumes; // volumes[] in volume-BVH leaf order
    std::vector<VolNode> volume_nodes;
    std::vector<float> volume_grids; // VolumePrim grid offsets index this pool
    Camera camera{};
    RenderParams params;
    std::vector<PostProcess> post;
    V3 world_min, world_max;
    uint64_t triangle_count = 0;     // after instance flattening
};

// Load a scene file. Throws json::ParseError / std::runtime_error on bad input.
HostScene load_scene(const std::string &path);

// Camera setup (builtin/btrc/builtin/camera/pinhole.cpp:55-77).
Camera make_pinhole(V3 eye, V3 dst, V3 up, float fov_y_deg, float w_over_h);

// Alias table construction (common/btrc/utils/math/alias.cpp:13-50).
std::vector<AliasEntry8> build_alias_table(const std::vector<float> &weights);

// Gaussian filter importance-sampling table, 256 x 256 cells over [-r, r]^2
// (builtin/btrc/builtin/film_filter/gaussian.cpp:27-52).
std::vector<AliasEntry8> build_gaussian_filter_table(float radius, float alpha);

// Load one OBJ file into triangle-soup shading data
// (common/btrc/utils/triangle_mesh_loader.cpp:16-150; polygons fan-triangulated).
HostGeometry load_obj(const std::string &filename, bool to_unit_cube);

} // namespace bt
