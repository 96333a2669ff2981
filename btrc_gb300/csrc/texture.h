// 2D texture evaluation shared by the kernels and the host (environment-map
// preprocessing): image textures sampled like a CUDA texture object with normalised
// coordinates (builtin/btrc/builtin/texture2d/array2d.cpp:17-29 over
// common/btrc/utils/cuda/texture.cpp:62-102), and postfix texture programs for the
// add / sub / mul / div and uv-transform textures (texture2d/math.cpp,
// texture2d/transform.cpp). Bilinear weights are exact here; the texture unit quantises
// them to 8 fractional bits.
#pragma once

#include "bmath.h"
#include "layout.h"

namespace bt {

struct TexTables
{
    const TexImage *images;
    const float *texels;     // 4 floats per texel
    const TexInstr *instr;
};

BT_HD V3 tex_texel(const float *texels, int64_t idx)
{
#ifdef __CUDA_ARCH__
    const float4 t = __ldg(reinterpret_cast<const float4 *>(texels) + idx);
    return V3(t.x, t.y, t.z);
#else
    const float *t = texels + idx * 4;
    return V3(t[0], t[1], t[2]);
#endif
}

// integer texel index under an address mode; false: outside a border-mode texture
BT_HD bool tex_index(int i, int n, int mode, int &out)
{
    if(mode == TEX_WRAP)
    {
        int m = i % n;
        out = m < 0 ? m + n : m;
        return true;
    }
    if(mode == TEX_MIRROR)
    {
        const int p = 2 * n;
        int m = i % p;
        m = m < 0 ? m + p : m;
        out = m < n ? m : p - 1 - m;
        return true;
    }
    if(mode == TEX_BORDER)
    {
        out = i;
        return i >= 0 && i < n;
    }
    out = i < 0 ? 0 : (i >= n ? n - 1 : i);
    return true;
}

// normalised coordinate under wrap / mirror (the others keep it)
BT_HD float tex_coord(float u, int mode)
{
    if(mode == TEX_WRAP)
        return u - floorf(u);
    if(mode == TEX_MIRROR)
    {
        const float f = floorf(u);
        const float r = u - f;
        const int k = static_cast<int>(f);
        return (k & 1) ? 1.0f - r : r;
    }
    return u;
}

BT_HD V3 tex_fetch(const TexImage &im, const float *texels, int x, int y)
{
    int ix, iy;
    const bool inx = tex_index(x, im.width, im.address_u, ix);
    const bool iny = tex_index(y, im.height, im.address_v, iy);
    if(!inx || !iny)
        return V3(im.border[0], im.border[1], im.border[2]);
    return tex_texel(texels, static_cast<int64_t>(im.offset) + static_cast<int64_t>(iy) * im.width + ix);
}

BT_HD V3 tex_sample_image(const TexImage &im, const float *texels, float u, float v)
{
    u = tex_coord(u, im.address_u);
    v = tex_coord(v, im.address_v);
    if(!(u == u) || !(v == v))
        return V3(0.0f);
    if(im.filter == 0)
    {
        const int x = static_cast<int>(floorf(fminf(fmaxf(u * im.width, -1.0e9f), 1.0e9f)));
        const int y = static_cast<int>(floorf(fminf(fmaxf(v * im.height, -1.0e9f), 1.0e9f)));
        return tex_fetch(im, texels, x, y);
    }
    const float xb = fminf(fmaxf(u * im.width - 0.5f, -1.0e9f), 1.0e9f);
    const float yb = fminf(fmaxf(v * im.height - 0.5f, -1.0e9f), 1.0e9f);
    const float fx = floorf(xb), fy = floorf(yb);
    const float ax = xb - fx, ay = yb - fy;
    const int x0 = static_cast<int>(fx), y0 = static_cast<int>(fy);
    const V3 t00 = tex_fetch(im, texels, x0, y0), t10 = tex_fetch(im, texels, x0 + 1, y0);
    const V3 t01 = tex_fetch(im, texels, x0, y0 + 1), t11 = tex_fetch(im, texels, x0 + 1, y0 + 1);
    return (t00 * (1.0f - ax) + t10 * ax) * (1.0f - ay) + (t01 * (1.0f - ax) + t11 * ax) * ay;
}

// run the program starting at instruction `prog` at texture coordinate (u, v)
BT_HD V3 tex_eval(const TexTables &T, int prog, float u, float v)
{
    V3 st[TEX_STACK];
    int sp = 0;
    for(int k = prog;; ++k)
    {
        const TexInstr &ins = T.instr[k];
        switch(ins.op)
        {
        case TEXOP_CONST:
            st[sp++] = V3(ins.a[0], ins.a[1], ins.a[2]);
            break;
        case TEXOP_SAMPLE:
        {
            const float uu = ins.a[0] * u + ins.a[1] * v + ins.a[2];
            const float vv = ins.a[3] * u + ins.a[4] * v + ins.a[5];
            st[sp++] = tex_sample_image(T.images[ins.image], T.texels, uu, vv);
            break;
        }
        case TEXOP_ADD:
            st[sp - 2] = st[sp - 2] + st[sp - 1];
            --sp;
            break;
        case TEXOP_SUB:
            st[sp - 2] = st[sp - 2] - st[sp - 1];
            --sp;
            break;
        case TEXOP_MUL:
            st[sp - 2] = st[sp - 2] * st[sp - 1];
            --sp;
            break;
        case TEXOP_DIV:
            st[sp - 2] = st[sp - 2] / st[sp - 1];
            --sp;
            break;
        default:
            return sp > 0 ? st[sp - 1] : V3(0.0f);
        }
    }
}

} // namespace bt
