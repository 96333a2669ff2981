#include "textures.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <filesystem>
#include <numeric>
#include <stdexcept>

#include "image_io.h"
#include "scene.h"
#include "texture.h"

namespace bt {

namespace {

using json::NodeP;

// 2x3 affine map of texture coordinates, rows (a0 a1 a2), (a3 a4 a5)
struct Affine2
{
    float a[6] = { 1, 0, 0, 0, 1, 0 };
};

// Mat3 product of the reference (common/btrc/utils/math/mat3.cpp) restricted to affine maps
Affine2 mul(const Affine2 &x, const Affine2 &y)
{
    Affine2 r;
    const float X[3][3] = { { x.a[0], x.a[1], x.a[2] }, { x.a[3], x.a[4], x.a[5] }, { 0, 0, 1 } };
    const float Y[3][3] = { { y.a[0], y.a[1], y.a[2] }, { y.a[3], y.a[4], y.a[5] }, { 0, 0, 1 } };
    for(int row = 0; row < 2; ++row)
        for(int col = 0; col < 3; ++col)
        {
            float s = 0;
            for(int k = 0; k < 3; ++k)
                s += X[row][k] * Y[k][col];
            r.a[row * 3 + col] = s;
        }
    return r;
}

float vec2_component(const NodeP &n, int i)
{
    if(n->is_array())
    {
        if(n->elems.size() == 1)
            return json::as_float(n->elems[0]);
        if(n->elems.size() != 2)
            throw std::runtime_error("two-component vector expected");
        return json::as_float(n->elems[i]);
    }
    return json::as_float(n);
}

// parse_transform2d (factory/btrc/factory/node/node.cpp:126-164)
Affine2 parse_transform2d(const NodeP &n)
{
    if(n->is_array())
    {
        Affine2 t;
        for(auto &e : n->elems)
            t = mul(parse_transform2d(e), t);
        return t;
    }
    Affine2 t;
    if(auto c = n->find("translate"))
    {
        t.a[2] = vec2_component(c, 0);
        t.a[5] = vec2_component(c, 1);
        return t;
    }
    if(auto c = n->find("rotate"))
    {
        const float rad = json::as_radian(c->child("angle"));
        const float s = std::sin(rad), co = std::cos(rad);
        t.a[0] = co; t.a[1] = -s; t.a[3] = s; t.a[4] = co;
        return t;
    }
    if(auto c = n->find("scale"))
    {
        t.a[0] = vec2_component(c, 0);
        t.a[4] = vec2_component(c, 1);
        return t;
    }
    if(auto c = n->find("inverse_u"); c && json::as_bool(c))
    {
        t.a[0] = -1; t.a[2] = 1;
        return t;
    }
    if(auto c = n->find("inverse_v"); c && json::as_bool(c))
    {
        t.a[4] = -1; t.a[5] = 1;
        return t;
    }
    if(auto c = n->find("swap_uv"); c && json::as_bool(c))
    {
        t.a[0] = 0; t.a[1] = 1; t.a[3] = 1; t.a[4] = 0;
        return t;
    }
    throw std::runtime_error("unknown transform2d type");
}

int address_mode(const NodeP &n, const char *key)
{
    auto c = n->find(key);
    const std::string s = c ? json::as_string(c) : "clamp";
    if(s == "clamp")
        return TEX_CLAMP;
    if(s == "mirror")
        return TEX_MIRROR;
    if(s == "wrap")
        return TEX_WRAP;
    if(s == "border")
        return TEX_BORDER;
    throw std::runtime_error("unknown address mode: " + s);
}

float srgb_to_linear(float c)
{
    return c <= 0.04045f ? c / 12.92f : std::pow((c + 0.055f) / 1.055f, 2.4f);
}

std::string resolve(const std::string &p, const std::string &scene_dir)
{
    std::string r = p;
    const std::string key = "$env{scene_directory}";
    for(size_t k = r.find(key); k != std::string::npos; k = r.find(key))
        r.replace(k, key.size(), scene_dir);
    std::filesystem::path fp(r);
    if(fp.is_relative())
        fp = std::filesystem::absolute(fp);
    return fp.lexically_normal().string();
}

// Array2DCreator (texture2d/array2d.cpp:37-45) with parse_texture_desc (description.cpp:28-80)
int load_array_image(TexStore &T, const NodeP &n)
{
    const std::string file = resolve(json::as_string(n->child("filename")), T.scene_dir);
    TexImage im{};
    im.address_u = address_mode(n, "address_mode_u");
    im.address_v = address_mode(n, "address_mode_v");
    (void)address_mode(n, "address_mode_w");
    const std::string filter = n->find("filter") ? json::as_string(n->child("filter")) : "linear";
    if(filter == "point")
        im.filter = 0;
    else if(filter == "linear")
        im.filter = 1;
    else
        throw std::runtime_error("unknown filter mode: " + filter);
    const bool srgb = json::bool_or(n, "srgb_to_linear", false);
    if(auto b = n->find("border"))
    {
        if(b->is_array())
        {
            if(b->elems.size() == 1)
                im.border[0] = im.border[1] = im.border[2] = im.border[3] = json::as_float(b->elems[0]);
            else if(b->elems.size() == 3)
                for(int c = 0; c < 3; ++c)
                    im.border[c] = json::as_float(b->elems[c]);
            else
                throw std::runtime_error("invalid border array size");
        }
        else if(b->is_value())
            im.border[0] = im.border[1] = im.border[2] = im.border[3] = json::as_float(b);
        else
            throw std::runtime_error("border: expect array or value node");
    }
    char key[512];
    std::snprintf(key, sizeof(key), "|%d|%d|%d|%d|%g|%g|%g|%g", im.address_u, im.address_v, im.filter, srgb ? 1 : 0,
                  im.border[0], im.border[1], im.border[2], im.border[3]);
    const std::string cache_key = file + key;
    auto it = T.image_cache.find(cache_key);
    if(it != T.image_cache.end())
        return it->second;
    LoadedImage img = load_image(file);
    im.width = img.width;
    im.height = img.height;
    if(T.texels.size() / 4 + img.texels.size() / 4 > static_cast<size_t>(INT32_MAX))
        throw std::runtime_error("texture texels exceed 2^31");
    im.offset = static_cast<int32_t>(T.texels.size() / 4);
    // the texture unit decodes sRGB for 8-bit formats only, before filtering
    if(srgb && !img.is_float)
        for(size_t i = 0; i < img.texels.size(); i += 4)
            for(int c = 0; c < 3; ++c)
                img.texels[i + c] = srgb_to_linear(img.texels[i + c]);
    T.texels.insert(T.texels.end(), img.texels.begin(), img.texels.end());
    T.images.push_back(im);
    const int id = static_cast<int>(T.images.size()) - 1;
    T.image_cache[cache_key] = id;
    return id;
}

bool constant_value(const NodeP &n, V3 &v)
{
    if(n->is_value() || n->is_array())
    {
        v = json::as_spectrum(n);
        return true;
    }
    if(json::as_string(n->child("type")) == "constant")
    {
        v = json::as_spectrum(n->child("value"));
        return true;
    }
    return false;
}

void emit(TexStore &T, const NodeP &n, const Affine2 &uvmap, std::vector<TexInstr> &code)
{
    TexInstr ins{};
    V3 c;
    if(constant_value(n, c))
    {
        ins.op = TEXOP_CONST;
        ins.a[0] = c.x; ins.a[1] = c.y; ins.a[2] = c.z;
        code.push_back(ins);
        return;
    }
    const std::string type = json::as_string(n->child("type"));
    if(type == "array")
    {
        ins.op = TEXOP_SAMPLE;
        ins.image = load_array_image(T, n);
        std::copy(uvmap.a, uvmap.a + 6, ins.a);
        code.push_back(ins);
        return;
    }
    if(type == "add" || type == "sub" || type == "mul" || type == "div")
    {
        emit(T, n->child("lhs"), uvmap, code);
        emit(T, n->child("rhs"), uvmap, code);
        ins.op = type == "add" ? TEXOP_ADD : type == "sub" ? TEXOP_SUB : type == "mul" ? TEXOP_MUL : TEXOP_DIV;
        code.push_back(ins);
        return;
    }
    if(type == "transform")
    {
        // TransformTexture2D::map_uv: the inner texture sees transform(uv)
        emit(T, n->child("tex"), mul(parse_transform2d(n->child("transform")), uvmap), code);
        return;
    }
    throw std::runtime_error("unsupported texture2d type '" + type + "'");
}

} // namespace

int compile_texture2d(TexStore &T, const NodeP &n, V3 &constant)
{
    if(constant_value(n, constant))
        return -1;
    std::vector<TexInstr> code;
    emit(T, n, Affine2{}, code);
    int depth = 0, max_depth = 0;
    for(const TexInstr &i : code)
    {
        depth += (i.op == TEXOP_CONST || i.op == TEXOP_SAMPLE) ? 1 : -1;
        max_depth = std::max(max_depth, depth);
    }
    if(max_depth > TEX_STACK)
        throw std::runtime_error("texture expression nested too deeply (more than 8 pending operands)");
    TexInstr end{};
    end.op = TEXOP_END;
    code.push_back(end);
    const int start = static_cast<int>(T.instr.size());
    T.instr.insert(T.instr.end(), code.begin(), code.end());
    return start;
}

void build_env_sampler(const TexStore &T, int prog, int lut_w, int lut_h, std::vector<float> &probs,
                       std::vector<AliasEntry8> &alias)
{
    const TexTables tables{ T.images.data(), T.texels.data(), T.instr.data() };
    constexpr int N = 256;
    const float PI_F = 3.14159265358979323846f;
    std::vector<float> lum(static_cast<size_t>(lut_w) * lut_h), area(lum.size());
    for(int yi = 0; yi < lut_h; ++yi)
        for(int xi = 0; xi < lut_w; ++xi)
        {
            const float x0 = static_cast<float>(xi) / lut_w, x1 = static_cast<float>(xi + 1) / lut_w;
            const float y0 = static_cast<float>(yi) / lut_h, y1 = static_cast<float>(yi + 1) / lut_h;
            float sum = 0.0f;
            for(int i = 0; i < N; ++i)
            {
                // hammersley2d (common/btrc/utils/math/hammersley.h)
                uint32_t bits = static_cast<uint32_t>(i);
                bits = (bits << 16u) | (bits >> 16u);
                bits = ((bits & 0x55555555u) << 1u) | ((bits & 0xAAAAAAAAu) >> 1u);
                bits = ((bits & 0x33333333u) << 2u) | ((bits & 0xCCCCCCCCu) >> 2u);
                bits = ((bits & 0x0F0F0F0Fu) << 4u) | ((bits & 0xF0F0F0F0u) >> 4u);
                bits = ((bits & 0x00FF00FFu) << 8u) | ((bits & 0xFF00FF00u) >> 8u);
                const float hx = static_cast<float>(i) / N, hy = bits * 2.3283064365386963e-10f;
                const float sx = 1.2f * hx - 0.1f, sy = 1.2f * hy - 0.1f;
                const float x = x0 + (x1 - x0) * sx, y = y0 + (y1 - y0) * sy;
                const V3 v = tex_eval(tables, prog, x, y);
                sum += 0.2126f * v.x + 0.7152f * v.y + 0.0722f * v.z;
            }
            const size_t k = static_cast<size_t>(yi) * lut_w + xi;
            lum[k] = sum / N;
            area[k] = std::fabs(2 * PI_F * (x1 - x0) * (std::cos(PI_F * y1) - std::cos(PI_F * y0)));
        }
    float lum_area = 0.0f, area_sum = 0.0f;
    for(size_t i = 0; i < lum.size(); ++i)
    {
        lum_area += lum[i] * area[i];
        area_sum += area[i];
    }
    const float avg = lum_area / area_sum;
    for(size_t i = 0; i < lum.size(); ++i)
        lum[i] = std::max(0.0f, area[i] * (lum[i] - avg));
    const float total = std::accumulate(lum.begin(), lum.end(), 0.0f);
    if(total > 1e-3f)
    {
        const float ratio = 1 / total;
        for(float &v : lum)
            v *= ratio;
    }
    probs = lum;
    if(total > 0)
        alias = build_alias_table(lum);
    else
    {
        // no tile above the mean (a uniform map): the reference's alias table over zeros
        // picks tile floor(n u), and every tile reports probability 0
        alias.resize(lum.size());
        for(size_t i = 0; i < lum.size(); ++i)
        {
            alias[i].accept = 1.0f;
            alias[i].alias = static_cast<uint32_t>(i);
        }
    }
}

} // namespace bt
