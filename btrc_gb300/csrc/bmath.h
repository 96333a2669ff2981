// Small host/device vector math shared by the host runtime and the CUDA kernels.
// Everything is plain FP32; operator order is written out so that host and
// device produce identical roundings where that matters (transforms, the
// watertight triangle test lives in traverse.cuh with explicit _rn intrinsics).
#pragma once

#include <cstdint>
#include <cmath>

#if defined(__CUDACC__)
#define BT_HD __host__ __device__ __forceinline__
#else
#define BT_HD inline
#endif

namespace bt {

constexpr float PI = 3.14159265358979323846f;
constexpr float MAX_FLOAT = 3.402823466e+38f;

struct V3
{
    float x, y, z;
    BT_HD V3() : x(0), y(0), z(0) {}
    BT_HD V3(float v) : x(v), y(v), z(v) {}
    BT_HD V3(float a, float b, float c) : x(a), y(b), z(c) {}
    BT_HD float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    BT_HD float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};

BT_HD V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
BT_HD V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
BT_HD V3 operator*(V3 a, V3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
BT_HD V3 operator/(V3 a, V3 b) { return V3(a.x / b.x, a.y / b.y, a.z / b.z); }
BT_HD V3 operator*(V3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
BT_HD V3 operator*(float s, V3 a) { return V3(a.x * s, a.y * s, a.z * s); }
BT_HD V3 operator/(V3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
BT_HD V3 operator-(V3 a) { return V3(-a.x, -a.y, -a.z); }
BT_HD V3 &operator+=(V3 &a, V3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
BT_HD V3 &operator*=(V3 &a, V3 b) { a.x *= b.x; a.y *= b.y; a.z *= b.z; return a; }
BT_HD V3 &operator*=(V3 &a, float s) { a.x *= s; a.y *= s; a.z *= s; return a; }

BT_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
BT_HD V3 cross(V3 a, V3 b)
{
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
BT_HD float length_square(V3 a) { return dot(a, a); }
BT_HD float length(V3 a) { return sqrtf(dot(a, a)); }
BT_HD V3 normalize(V3 a) { return a * (1.0f / length(a)); }
BT_HD V3 vmin(V3 a, V3 b) { return V3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
BT_HD V3 vmax(V3 a, V3 b) { return V3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
BT_HD float max_comp(V3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
BT_HD bool is_zero(V3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
BT_HD float saturate(float v) { return fminf(1.0f, fmaxf(0.0f, v)); }

// IEEE-rounded reciprocal. The shading translation unit is compiled with approximate
// division; code that must match the oracle bit for bit (sampler, traversal setup) uses
// this instead of 1.0f / x.
BT_HD float rcp_rn(float x)
{
#if defined(__CUDA_ARCH__)
    return __frcp_rn(x);
#else
    return 1.0f / x;
#endif
}

// sin(pi x) and cos(pi x). Every angle the tracer samples is a fraction of pi, and on
// the device sincospif reduces such arguments exactly, so it needs none of the large-
// argument code that sinf / cosf carry at each call site.
BT_HD void sincos_pi(float x, float &s, float &c)
{
#if defined(__CUDA_ARCH__)
    sincospif(x, &s, &c);
#else
    s = std::sin(PI * x);
    c = std::cos(PI * x);
#endif
}

BT_HD float cos_pi(float x)
{
#if defined(__CUDA_ARCH__)
    return cospif(x);
#else
    return std::cos(PI * x);
#endif
}
BT_HD float clampf(float v, float lo, float hi) { return fminf(hi, fmaxf(lo, v)); }
BT_HD float lerpf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
BT_HD V3 lerp3(V3 a, V3 b, float t) { return a * (1.0f - t) + b * t; }

// Rec.709 luminance (reference: core/btrc/core/spectrum.cpp:35-38)
BT_HD float luminance(V3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

#if defined(__CUDA_ARCH__)
BT_HD bool all_finite(V3 v) { return isfinite(v.x) && isfinite(v.y) && isfinite(v.z); }
#else
BT_HD bool all_finite(V3 v) { return std::isfinite(v.x) && std::isfinite(v.y) && std::isfinite(v.z); }
#endif

BT_HD uint32_t f2u(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    union { float f; uint32_t u; } c; c.f = f; return c.u;
#endif
}
BT_HD float u2f(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    union { float f; uint32_t u; } c; c.u = u; return c.f;
#endif
}
BT_HD int32_t f2i_bits(float f) { return (int32_t)f2u(f); }
BT_HD float i2f_bits(int32_t i) { return u2f((uint32_t)i); }

// Orthonormal frame (reference: common/btrc/utils/cmath/cframe.cpp:13-83)
struct Frame
{
    V3 x, y, z;
    BT_HD Frame() : x(1, 0, 0), y(0, 1, 0), z(0, 0, 1) {}
    BT_HD Frame(V3 a, V3 b, V3 c) : x(normalize(a)), y(normalize(b)), z(normalize(c)) {}

    BT_HD static Frame from_z(V3 zz)
    {
        V3 nz = normalize(zz), ny;
        if(1.0f - fabsf(nz.x) < 0.1f)
            ny = cross(nz, V3(0, 1, 0));
        else
            ny = cross(nz, V3(1, 0, 0));
        // x = z cross y, as CFrame::from_z builds it (common/btrc/utils/cmath/cframe.cpp:52-64)
        return Frame(cross(nz, ny), ny, nz);
    }
    BT_HD V3 local_to_global(V3 l) const { return x * l.x + y * l.y + z * l.z; }
    BT_HD V3 global_to_local(V3 g) const { return V3(dot(g, x), dot(g, y), dot(g, z)); }
    BT_HD Frame rotate_to_new_z(V3 nz) const
    {
        V3 nx = cross(y, nz);
        V3 ny = cross(nz, nx);
        return Frame(nx, ny, nz);
    }
    BT_HD bool in_positive_z_hemisphere(V3 v) const { return dot(v, z) > 0; }
};

// 3x4 affine matrix, row major, used for instance transforms.
// apply_to_point/vector follow common/btrc/utils/cmath/ctransform.cpp (left to right sums).
struct Affine
{
    float m[12];
    BT_HD V3 point(V3 p) const
    {
        return V3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3],
                  m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
                  m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
    }
    BT_HD V3 vector(V3 v) const
    {
        return V3(m[0] * v.x + m[1] * v.y + m[2] * v.z,
                  m[4] * v.x + m[5] * v.y + m[6] * v.z,
                  m[8] * v.x + m[9] * v.y + m[10] * v.z);
    }
    // normal transform uses the inverse's transpose: this matrix must hold the inverse
    BT_HD V3 normal_from_inverse(V3 n) const
    {
        return V3(m[0] * n.x + m[4] * n.y + m[8] * n.z,
                  m[1] * n.x + m[5] * n.y + m[9] * n.z,
                  m[2] * n.x + m[6] * n.y + m[10] * n.z);
    }
};

} // namespace bt
