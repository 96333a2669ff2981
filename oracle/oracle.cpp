// ORACLE — test infrastructure only. A CPU restatement of the reference (AirGuanZ/Btrc)
// hot path, used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline as the
// checker. The product (btrc_gb300) never includes, links or calls this file.
//
// Parity status: the reference cannot be built or run (its eDSL submodule and the OptiX
// SDK are absent), so this restatement is pinned where a published or vendored answer
// exists: PCG32 against O'Neill's published pcg32 demo output, closest-hit traversal
// against the vendored madmann91/bvh library compiled from the reference tree
// (oracle/ref_bvh.cpp), and the samplers/BSDFs against closed-form properties in the tests.
// Elsewhere parity is unpinned: the restatement follows the reference source line by line.
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fPIC -shared -pthread (oracle/build.py).
// -ffp-contract=off matters: the watertight test must round every product and sum
// separately, exactly like the CUDA kernel's explicitly rounded intrinsics.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>
#include <vector>

namespace orc {

constexpr float PIf = 3.14159265358979323846f;
constexpr float FMAX = std::numeric_limits<float>::max();

template<class T>
struct V
{
    T x, y, z;
    V() : x(0), y(0), z(0) {}
    V(T v) : x(v), y(v), z(v) {}
    V(T a, T b, T c) : x(a), y(b), z(c) {}
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template<class T> V<T> operator+(V<T> a, V<T> b) { return V<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template<class T> V<T> operator-(V<T> a, V<T> b) { return V<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template<class T> V<T> operator*(V<T> a, V<T> b) { return V<T>(a.x * b.x, a.y * b.y, a.z * b.z); }
template<class T> V<T> operator*(V<T> a, T s) { return V<T>(a.x * s, a.y * s, a.z * s); }
template<class T> V<T> operator*(T s, V<T> a) { return V<T>(a.x * s, a.y * s, a.z * s); }
template<class T> V<T> operator/(V<T> a, T s) { return V<T>(a.x / s, a.y / s, a.z / s); }
template<class T> V<T> operator/(V<T> a, V<T> b) { return V<T>(a.x / b.x, a.y / b.y, a.z / b.z); }
template<class T> V<T> operator-(V<T> a) { return V<T>(-a.x, -a.y, -a.z); }
template<class T> T dot(V<T> a, V<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template<class T> V<T> cross(V<T> a, V<T> b) { return V<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
template<class T> T len(V<T> a) { return std::sqrt(dot(a, a)); }
template<class T> V<T> nrm(V<T> a) { return a * (T(1) / len(a)); }
template<class T> bool zero3(V<T> a) { return a.x == 0 && a.y == 0 && a.z == 0; }
template<class T> T lum(V<T> c) { return T(0.2126) * c.x + T(0.7152) * c.y + T(0.0722) * c.z; }
template<class T> V<T> lerp(V<T> a, V<T> b, T t) { return a * (T(1) - t) + b * t; }
template<class T> T lerp1(T a, T b, T t) { return a * (T(1) - t) + b * t; }
template<class T> T clampv(T v, T lo, T hi) { return std::min(hi, std::max(lo, v)); }
template<class T> T sq(T v) { return v * v; }

using V3f = V<float>;

// ------------------------------------------------------------------ frames (cframe.cpp:13-83)

template<class T>
struct Frame
{
    V<T> x, y, z;
    Frame() : x(1, 0, 0), y(0, 1, 0), z(0, 0, 1) {}
    Frame(V<T> a, V<T> b, V<T> c) : x(nrm(a)), y(nrm(b)), z(nrm(c)) {}
    static Frame from_z(V<T> zz)
    {
        V<T> nz = nrm(zz), ny;
        if(T(1) - std::abs(nz.x) < T(0.1))
            ny = cross(nz, V<T>(0, 1, 0));
        else
            ny = cross(nz, V<T>(1, 0, 0));
        // x = z cross y (common/btrc/utils/cmath/cframe.cpp:52-64)
        return Frame(cross(nz, ny), ny, nz);
    }
    V<T> l2g(V<T> l) const { return x * l.x + y * l.y + z * l.z; }
    V<T> g2l(V<T> g) const { return V<T>(dot(g, x), dot(g, y), dot(g, z)); }
    Frame rotate_to_new_z(V<T> nz) const
    {
        V<T> nx = cross(y, nz);
        V<T> ny = cross(nz, nx);
        return Frame(nx, ny, nz);
    }
    bool upper(V<T> v) const { return dot(v, z) > 0; }
};

// ------------------------------------------------------------------ watertight triangle test
// Woop, Benthin, Wald (JCGT 2013), FP32, every operation rounded separately.

struct WRay
{
    float o[3], d[3];
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

inline WRay make_wray(const float *o, const float *d)
{
    WRay r;
    for(int k = 0; k < 3; ++k)
    {
        r.o[k] = o[k];
        r.d[k] = d[k];
    }
    const float ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
    int kz = (ax >= ay) ? ((ax >= az) ? 0 : 2) : ((ay >= az) ? 1 : 2);
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    if(d[kz] < 0.0f)
        std::swap(kx, ky);
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = d[kx] / d[kz];
    r.Sy = d[ky] / d[kz];
    r.Sz = 1.0f / d[kz];
    return r;
}

// returns true with t, b1 (weight of v1), b2 (weight of v2) when 0 < t <= tmax
inline bool watertight(const WRay &r, const float *v0, const float *v1, const float *v2, float tmax, float &t,
                       float &b1, float &b2)
{
    const float A[3] = { v0[0] - r.o[0], v0[1] - r.o[1], v0[2] - r.o[2] };
    const float B[3] = { v1[0] - r.o[0], v1[1] - r.o[1], v1[2] - r.o[2] };
    const float Cc[3] = { v2[0] - r.o[0], v2[1] - r.o[1], v2[2] - r.o[2] };
    const float Ax = A[r.kx] - r.Sx * A[r.kz];
    const float Ay = A[r.ky] - r.Sy * A[r.kz];
    const float Bx = B[r.kx] - r.Sx * B[r.kz];
    const float By = B[r.ky] - r.Sy * B[r.kz];
    const float Cx = Cc[r.kx] - r.Sx * Cc[r.kz];
    const float Cy = Cc[r.ky] - r.Sy * Cc[r.kz];
    float U = Cx * By - Cy * Bx;
    float Vv = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if(U == 0.0f || Vv == 0.0f || W == 0.0f)
    {
        U = static_cast<float>(static_cast<double>(Cx) * By - static_cast<double>(Cy) * Bx);
        Vv = static_cast<float>(static_cast<double>(Ax) * Cy - static_cast<double>(Ay) * Cx);
        W = static_cast<float>(static_cast<double>(Bx) * Ay - static_cast<double>(By) * Ax);
    }
    if((U < 0.0f || Vv < 0.0f || W < 0.0f) && (U > 0.0f || Vv > 0.0f || W > 0.0f))
        return false;
    const float det = (U + Vv) + W;
    if(det == 0.0f)
        return false;
    const float Az = r.Sz * A[r.kz];
    const float Bz = r.Sz * B[r.kz];
    const float Cz = r.Sz * Cc[r.kz];
    const float T = (U * Az + Vv * Bz) + W * Cz;
    const float rcp = 1.0f / det;
    const float tt = T * rcp;
    if(!(tt > 0.0f && tt <= tmax))
        return false;
    t = tt;
    b1 = Vv * rcp;
    b2 = W * rcp;
    return true;
}

// ------------------------------------------------------------------ oracle BVH (binary, SAH)

struct Box
{
    float lo[3] = { FMAX, FMAX, FMAX }, hi[3] = { -FMAX, -FMAX, -FMAX };
    void grow(const float *p)
    {
        for(int k = 0; k < 3; ++k)
        {
            lo[k] = std::min(lo[k], p[k]);
            hi[k] = std::max(hi[k], p[k]);
        }
    }
    void grow(const Box &b)
    {
        for(int k = 0; k < 3; ++k)
        {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    double area() const
    {
        if(lo[0] > hi[0])
            return 0;
        double dx = double(hi[0]) - lo[0], dy = double(hi[1]) - lo[1], dz = double(hi[2]) - lo[2];
        return 2 * (dx * dy + dy * dz + dz * dx);
    }
};

struct Node
{
    Box box;
    int left = -1, right = -1;
    uint32_t first = 0, count = 0;
};

struct Bvh
{
    std::vector<float> tri;       // 9 floats per triangle, leaf order
    std::vector<uint32_t> ids;    // inst, prim per triangle, leaf order
    std::vector<Node> nodes;

    void build(const float *tris, const uint32_t *idsin, uint64_t n)
    {
        std::vector<Box> boxes(n);
        std::vector<float> cen(n * 3);
        std::vector<uint32_t> idx(n);
        for(uint64_t i = 0; i < n; ++i)
        {
            for(int v = 0; v < 3; ++v)
                boxes[i].grow(tris + i * 9 + v * 3);
            for(int k = 0; k < 3; ++k)
                cen[i * 3 + k] = 0.5f * (boxes[i].lo[k] + boxes[i].hi[k]);
            idx[i] = static_cast<uint32_t>(i);
        }
        nodes.clear();
        nodes.reserve(2 * n + 1);
        nodes.emplace_back();
        if(n > 0)
            split(0, 0, static_cast<uint32_t>(n), boxes, cen, idx, 0);
        tri.resize(n * 9);
        ids.resize(n * 2);
        for(uint64_t i = 0; i < n; ++i)
        {
            std::memcpy(&tri[i * 9], tris + idx[i] * 9, 9 * sizeof(float));
            ids[i * 2] = idsin[idx[i] * 2];
            ids[i * 2 + 1] = idsin[idx[i] * 2 + 1];
        }
    }

    void split(int ni, uint32_t b, uint32_t e, const std::vector<Box> &boxes, const std::vector<float> &cen,
               std::vector<uint32_t> &idx, int depth)
    {
        Box box, cb;
        for(uint32_t i = b; i < e; ++i)
        {
            box.grow(boxes[idx[i]]);
            cb.grow(&cen[idx[i] * 3]);
        }
        nodes[ni].box = box;
        const uint32_t n = e - b;
        if(n <= 4 || depth > 60)
        {
            nodes[ni].first = b;
            nodes[ni].count = n;
            return;
        }
        constexpr int NB = 16;
        double best = std::numeric_limits<double>::infinity();
        int ba = -1, bb = -1;
        for(int a = 0; a < 3; ++a)
        {
            if(!(cb.hi[a] > cb.lo[a]))
                continue;
            const double sc = NB / (double(cb.hi[a]) - cb.lo[a]);
            Box bins[NB];
            uint32_t cnt[NB] = {};
            for(uint32_t i = b; i < e; ++i)
            {
                int k = std::min(NB - 1, std::max(0, int((cen[idx[i] * 3 + a] - double(cb.lo[a])) * sc)));
                bins[k].grow(boxes[idx[i]]);
                ++cnt[k];
            }
            for(int s = 0; s < NB - 1; ++s)
            {
                Box l, r;
                uint32_t nl = 0, nr = 0;
                for(int k = 0; k <= s; ++k)
                {
                    l.grow(bins[k]);
                    nl += cnt[k];
                }
                for(int k = s + 1; k < NB; ++k)
                {
                    r.grow(bins[k]);
                    nr += cnt[k];
                }
                if(!nl || !nr)
                    continue;
                const double c = l.area() * nl + r.area() * nr;
                if(c < best)
                {
                    best = c;
                    ba = a;
                    bb = s;
                }
            }
        }
        uint32_t mid;
        if(ba < 0)
            mid = b + n / 2;
        else
        {
            const double sc = NB / (double(cb.hi[ba]) - cb.lo[ba]);
            auto it = std::partition(idx.begin() + b, idx.begin() + e, [&](uint32_t p) {
                int k = std::min(NB - 1, std::max(0, int((cen[p * 3 + ba] - double(cb.lo[ba])) * sc)));
                return k <= bb;
            });
            mid = static_cast<uint32_t>(it - idx.begin());
            if(mid == b || mid == e)
                mid = b + n / 2;
        }
        const int l = static_cast<int>(nodes.size());
        nodes.emplace_back();
        nodes.emplace_back();
        nodes[ni].left = l;
        nodes[ni].right = l + 1;
        split(l, b, mid, boxes, cen, idx, depth + 1);
        split(l + 1, mid, e, boxes, cen, idx, depth + 1);
    }

    // conservative slab test in FP64
    static bool slab(const Box &bx, const double *o, const double *inv, double tmax, double &tnear)
    {
        double t0 = 0.0, t1 = tmax;
        for(int k = 0; k < 3; ++k)
        {
            double a = (double(bx.lo[k]) - o[k]) * inv[k];
            double b = (double(bx.hi[k]) - o[k]) * inv[k];
            if(a > b)
                std::swap(a, b);
            t0 = std::max(t0, a);
            t1 = std::min(t1, b);
        }
        tnear = t0;
        return t0 <= t1 * (1 + 1e-6) + 1e-30;
    }

    struct Hit
    {
        bool hit = false;
        float t = 0, b1 = 0, b2 = 0;
        uint32_t inst = 0, prim = 0;
    };

    Hit closest(const float *o, const float *d, float t1) const
    {
        Hit best;
        best.t = t1;
        if(nodes.empty() || tri.empty())
            return best;
        const WRay wr = make_wray(o, d);
        double od[3], inv[3];
        for(int k = 0; k < 3; ++k)
        {
            od[k] = o[k];
            inv[k] = 1.0 / (std::fabs(d[k]) < 1e-30 ? std::copysign(1e-30, d[k]) : double(d[k]));
        }
        int stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while(sp)
        {
            const Node &nd = nodes[stack[--sp]];
            double tn;
            if(!slab(nd.box, od, inv, double(best.t), tn))
                continue;
            if(nd.left < 0)
            {
                for(uint32_t i = nd.first; i < nd.first + nd.count; ++i)
                {
                    float t, b1, b2;
                    if(watertight(wr, &tri[i * 9], &tri[i * 9 + 3], &tri[i * 9 + 6], best.t, t, b1, b2))
                    {
                        const uint32_t inst = ids[i * 2], prim = ids[i * 2 + 1];
                        bool better = !best.hit || t < best.t ||
                                      (t == best.t && (inst < best.inst || (inst == best.inst && prim < best.prim)));
                        if(better)
                        {
                            best.hit = true;
                            best.t = t;
                            best.b1 = b1;
                            best.b2 = b2;
                            best.inst = inst;
                            best.prim = prim;
                        }
                    }
                }
                continue;
            }
            stack[sp++] = nd.left;
            stack[sp++] = nd.right;
        }
        return best;
    }

    bool any(const float *o, const float *d, float t1) const
    {
        if(nodes.empty() || tri.empty())
            return false;
        const WRay wr = make_wray(o, d);
        double od[3], inv[3];
        for(int k = 0; k < 3; ++k)
        {
            od[k] = o[k];
            inv[k] = 1.0 / (std::fabs(d[k]) < 1e-30 ? std::copysign(1e-30, d[k]) : double(d[k]));
        }
        int stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while(sp)
        {
            const Node &nd = nodes[stack[--sp]];
            double tn;
            if(!slab(nd.box, od, inv, double(t1), tn))
                continue;
            if(nd.left < 0)
            {
                for(uint32_t i = nd.first; i < nd.first + nd.count; ++i)
                {
                    float t, b1, b2;
                    if(watertight(wr, &tri[i * 9], &tri[i * 9 + 3], &tri[i * 9 + 6], t1, t, b1, b2))
                        return true;
                }
                continue;
            }
            stack[sp++] = nd.left;
            stack[sp++] = nd.right;
        }
        return false;
    }
};

template<class F>
void parallel_for(uint64_t n, int threads, F &&f)
{
    if(threads <= 0)
        threads = std::max(1u, std::thread::hardware_concurrency());
    std::atomic<uint64_t> next{ 0 };
    const uint64_t chunk = 256;
    auto work = [&] {
        for(;;)
        {
            const uint64_t b = next.fetch_add(chunk);
            if(b >= n)
                break;
            const uint64_t e = std::min(n, b + chunk);
            for(uint64_t i = b; i < e; ++i)
                f(i);
        }
    };
    std::vector<std::thread> pool;
    for(int k = 1; k < threads; ++k)
        pool.emplace_back(work);
    work();
    for(auto &t : pool)
        t.join();
}

// ------------------------------------------------------------------ samplers
// independent.cpp:11-24 (PCG32 seeded with murmur64A(pixel), advanced by sample*65536),
// halton.cpp:46-116 and low_discrepancy.cpp:10-99.

constexpr uint64_t PCG_MULT = 6364136223846793005ull;
constexpr uint64_t PCG_STREAM = 0xda3e39cb94b95bdbull;
constexpr float ONE_M_EPS = 0x1.fffffep-1f;

struct Pcg
{
    uint64_t state = 0, inc = 1;
    uint32_t next()
    {
        const uint64_t old = state;
        state = old * PCG_MULT + inc;
        const uint32_t xs = static_cast<uint32_t>(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = static_cast<uint32_t>(old >> 59u);
        return (xs >> rot) | (xs << ((0u - rot) & 31u));
    }
    void seed(uint64_t initstate, uint64_t initseq)
    {
        state = 0;
        inc = (initseq << 1u) | 1u;
        next();
        state += initstate;
        next();
    }
    void advance(uint64_t delta)
    {
        uint64_t cm = PCG_MULT, cp = inc, am = 1, ap = 0;
        while(delta)
        {
            if(delta & 1)
            {
                am *= cm;
                ap = ap * cm + cp;
            }
            cp = (cm + 1) * cp;
            cm *= cm;
            delta >>= 1;
        }
        state = am * state + ap;
    }
    float uniform()
    {
        const float v = static_cast<float>(next()) * 0x1p-32f;
        return std::min(v, ONE_M_EPS);
    }
};

inline uint64_t murmur64a(const uint8_t *key, uint64_t len, uint64_t seed)
{
    const uint64_t m = 0xc6a4a7935bd1e995ull;
    const int r = 47;
    uint64_t h = seed ^ (len * m);
    const uint8_t *end = key + 8 * (len / 8);
    while(key != end)
    {
        uint64_t k;
        std::memcpy(&k, key, 8);
        key += 8;
        k *= m;
        k ^= k >> r;
        k *= m;
        h ^= k;
        h *= m;
    }
    switch(len & 7)
    {
    case 7: h ^= uint64_t(key[6]) << 48; [[fallthrough]];
    case 6: h ^= uint64_t(key[5]) << 40; [[fallthrough]];
    case 5: h ^= uint64_t(key[4]) << 32; [[fallthrough]];
    case 4: h ^= uint64_t(key[3]) << 24; [[fallthrough]];
    case 3: h ^= uint64_t(key[2]) << 16; [[fallthrough]];
    case 2: h ^= uint64_t(key[1]) << 8; [[fallthrough]];
    case 1: h ^= uint64_t(key[0]); h *= m;
    }
    h ^= h >> r;
    h *= m;
    h ^= h >> r;
    return h;
}

inline uint64_t mix_bits(uint64_t v)
{
    v ^= v >> 31;
    v *= 0x7fb5d329728ea185ull;
    v ^= v >> 27;
    v *= 0x81dadef4bc2dd44dull;
    v ^= v >> 33;
    return v;
}

inline uint32_t perm_element(uint32_t i, uint32_t l, uint32_t p)
{
    uint32_t w = l - 1;
    w |= w >> 1;
    w |= w >> 2;
    w |= w >> 4;
    w |= w >> 8;
    w |= w >> 16;
    for(;;)
    {
        i ^= p;
        i *= 0xe170893du;
        i ^= p >> 16;
        i ^= (i & w) >> 4;
        i ^= p >> 8;
        i *= 0x0929eb3fu;
        i ^= p >> 23;
        i ^= (i & w) >> 1;
        i *= 1u | p >> 27;
        i *= 0x6935fa69u;
        i ^= (i & w) >> 11;
        i *= 0x74dcb303u;
        i ^= (i & w) >> 2;
        i *= 0x9e501cc3u;
        i ^= (i & w) >> 2;
        i *= 0xc860a3dfu;
        i &= w;
        i ^= i >> 5;
        if(i < l)
            break;
    }
    return (i + p) % l;
}

struct Primes
{
    uint32_t v[1000];
    Primes()
    {
        int n = 0;
        for(uint32_t c = 2; n < 1000; ++c)
        {
            bool ok = true;
            for(int k = 0; k < n && v[k] * v[k] <= c; ++k)
                if(c % v[k] == 0)
                {
                    ok = false;
                    break;
                }
            if(ok)
                v[n++] = c;
        }
    }
};
static const Primes PRIMES;

inline float owen_radical_inverse(int base_index, uint64_t a, uint64_t hash)
{
    const uint64_t base = PRIMES.v[base_index];
    const float inv_base = 1.0f / static_cast<float>(base);
    float inv_base_m = 1.0f;
    uint64_t reversed = 0;
    while(1.0f - inv_base_m < 1)
    {
        const uint64_t next = a / base;
        uint64_t digit = a - next * base;
        const uint64_t digit_hash = mix_bits(hash ^ reversed);
        digit = perm_element(static_cast<uint32_t>(digit), static_cast<uint32_t>(base), static_cast<uint32_t>(digit_hash));
        reversed = reversed * base + digit;
        inv_base_m = inv_base_m * inv_base;
        a = next;
    }
    return std::min(inv_base_m * static_cast<float>(reversed), ONE_M_EPS);
}

inline uint64_t inverse_radical_inverse(uint64_t inverse, uint64_t base, int digits)
{
    uint64_t index = 0;
    for(int i = 0; i < digits; ++i)
    {
        const uint64_t digit = inverse % base;
        inverse /= base;
        index = index * base + digit;
    }
    return index;
}

inline int64_t modi(int64_t a, int64_t b)
{
    const int64_t r = a - a / b * b;
    return r < 0 ? r + b : r;
}

inline void egcd(uint64_t a, uint64_t b, int64_t *x, int64_t *y)
{
    if(b == 0)
    {
        *x = 1;
        *y = 0;
        return;
    }
    int64_t d = a / b, xp, yp;
    egcd(b, a % b, &xp, &yp);
    *x = yp;
    *y = xp - d * yp;
}

struct Sampler
{
    int type = 0;  // 0 independent, 1 halton
    Pcg pcg;
    uint32_t dim = 0;
    uint64_t index = 0;

    struct HC
    {
        int scale[2], exp[2], mult[2], stride;
    };
    static HC consts(int w, int h)
    {
        HC c{};
        const int res[2] = { w, h };
        for(int i = 0; i < 2; ++i)
        {
            const int base = i == 0 ? 2 : 3;
            int s = 1, e = 0;
            while(s < std::min(res[i], 128))
            {
                s *= base;
                ++e;
            }
            c.scale[i] = s;
            c.exp[i] = e;
        }
        int64_t x, y;
        egcd(c.scale[1], c.scale[0], &x, &y);
        c.mult[0] = static_cast<int>(modi(x, c.scale[0]));
        egcd(c.scale[0], c.scale[1], &x, &y);
        c.mult[1] = static_cast<int>(modi(x, c.scale[1]));
        c.stride = c.scale[0] * c.scale[1];
        return c;
    }

    void init(int t, const HC &hc, uint32_t px, uint32_t py, uint32_t sample)
    {
        type = t;
        if(t == 0)
        {
            uint8_t buf[8];
            std::memcpy(buf, &px, 4);
            std::memcpy(buf + 4, &py, 4);
            pcg.seed(murmur64a(buf, 8, 0), PCG_STREAM);
            pcg.advance(static_cast<uint64_t>(sample) * 65536u);
            return;
        }
        index = 0;
        if(hc.stride > 1)
        {
            const uint64_t pm[2] = { px % 128u, py % 128u };
            for(int i = 0; i < 2; ++i)
            {
                const uint64_t off = inverse_radical_inverse(pm[i], i == 0 ? 2 : 3, hc.exp[i]);
                index = index + off * static_cast<uint64_t>((hc.stride / hc.scale[i]) * hc.mult[i]);
            }
            index = index % static_cast<uint64_t>(hc.stride);
        }
        index = index + static_cast<uint64_t>(sample) * static_cast<uint64_t>(hc.stride);
        dim = 2;
    }
    // the 16-byte state as the GPU stores it: independent (PCG state, inc), halton (index, dim)
    uint64_t word_a() const { return type == 0 ? pcg.state : index; }
    uint64_t word_b() const { return type == 0 ? pcg.inc : static_cast<uint64_t>(dim); }
    float halton(uint32_t d) const
    {
        return owen_radical_inverse(static_cast<int>(d), index, mix_bits(static_cast<uint64_t>(1u + (d << 4))));
    }
    float get1d()
    {
        if(type == 0)
            return pcg.uniform();
        if(dim >= 1000)
            dim = 2;
        const float v = halton(dim);
        dim += 1;
        return v;
    }
    void get3d(float &a, float &b, float &c)
    {
        if(type == 0)
        {
            a = pcg.uniform();
            b = pcg.uniform();
            c = pcg.uniform();
            return;
        }
        if(dim + 2 >= 1000)
            dim = 2;
        a = halton(dim);
        b = halton(dim + 1);
        c = halton(dim + 2);
        dim += 3;
    }
};

// ------------------------------------------------------------------ alias tables (alias.cpp:13-50)

struct Alias
{
    std::vector<float> accept;
    std::vector<uint32_t> other;
    void init(const std::vector<float> &p)
    {
        double s = 0;
        for(float v : p)
            s += v;
        const float ratio = static_cast<float>(p.size()) / static_cast<float>(s);
        accept.resize(p.size());
        other.resize(p.size());
        std::vector<uint32_t> overs, unders;
        for(uint32_t i = 0; i < p.size(); ++i)
        {
            accept[i] = p[i] * ratio;
            other[i] = i;
            if(accept[i] > 1)
                overs.push_back(i);
            else if(accept[i] < 1)
                unders.push_back(i);
        }
        while(!overs.empty() && !unders.empty())
        {
            const uint32_t o = overs.back(), u = unders.back();
            overs.pop_back();
            unders.pop_back();
            accept[o] -= 1 - accept[u];
            other[u] = o;
            if(accept[o] > 1)
                overs.push_back(o);
            else if(accept[o] < 1)
                unders.push_back(o);
        }
        for(auto i : overs)
            accept[i] = 1;
        for(auto i : unders)
            accept[i] = 1;
    }
    uint32_t sample(float u) const
    {
        const uint32_t n = static_cast<uint32_t>(accept.size());
        const float nu = static_cast<float>(n) * u;
        const uint32_t i = std::min(static_cast<uint32_t>(nu), n - 1);
        const float s = nu - static_cast<float>(i);
        return s <= accept[i] ? i : other[i];
    }
};

// ------------------------------------------------------------------ BSDFs (templated: FP32 render, FP64 check)

template<class T> struct CS
{
    V<T> f, dir;
    T pdf = 0;
    bool delta = false;
};

template<class T> T PI_T() { return T(3.14159265358979323846); }

// sin(pi x) and cos(pi x), as the kernels evaluate sampled angles (sincospif): computed
// in double and rounded once
template<class T> void sincos_pi(T x, T &s, T &c)
{
    const double a = 3.14159265358979323846 * static_cast<double>(x);
    s = static_cast<T>(std::sin(a));
    c = static_cast<T>(std::cos(a));
}
template<class T> T cos_pi(T x) { return static_cast<T>(std::cos(3.14159265358979323846 * static_cast<double>(x))); }

template<class T> V<T> hemi_zw(T u1, T u2)
{
    T sx = 0, sy = 0;
    u1 = T(2) * u1 - T(1);
    u2 = T(2) * u2 - T(1);
    if(u1 != 0 || u2 != 0)
    {
        T theta, r;  // in units of pi
        if(std::abs(u1) > std::abs(u2))
        {
            r = u1;
            theta = T(0.25) * (u2 / u1);
        }
        else
        {
            r = u2;
            theta = T(0.5) - T(0.25) * (u1 / u2);
        }
        T st, ct;
        sincos_pi(theta, st, ct);
        sx = r * ct;
        sy = r * st;
    }
    return V<T>(sx, sy, std::sqrt(std::max(T(0), T(1) - (sx * sx + sy * sy))));
}
template<class T> T pdf_hemi_zw(V<T> v) { return v.z >= 0 ? v.z / PI_T<T>() : T(0); }
template<class T> T cos2sin(T c) { return std::sqrt(std::max(T(0), T(1) - c * c)); }
template<class T> T tan_th(V<T> w)
{
    T t = T(1) - w.z * w.z;
    return t > 0 ? std::sqrt(t) / w.z : T(0);
}
template<class T> T phi_of(V<T> w)
{
    T r = 0;
    if(w.x != 0 || w.y != 0)
    {
        r = std::atan2(w.y, w.x);
        if(r < 0)
            r += 2 * PI_T<T>();
    }
    return r;
}
template<class T> T diel_fresnel(T ei, T eo, T ci)
{
    if(ci < 0)
    {
        std::swap(ei, eo);
        ci = -ci;
    }
    const T si = std::sqrt(std::max(T(0), T(1) - ci * ci));
    const T st = eo / ei * si;
    if(st >= 1)
        return T(1);
    const T ct = std::sqrt(std::max(T(0), T(1) - st * st));
    const T para = (ei * ci - eo * ct) / (ei * ci + eo * ct);
    const T perp = (eo * ci - ei * ct) / (eo * ci + ei * ct);
    return T(0.5) * (para * para + perp * perp);
}
template<class T> T schlick1(T r0, T c)
{
    T t = T(1) - c, t2 = t * t;
    return r0 + (T(1) - r0) * (t2 * t2 * t);
}
template<class T> V<T> schlick3(V<T> r0, T c)
{
    T t = T(1) - c, t2 = t * t, t5 = t2 * t2 * t;
    return r0 + (V<T>(T(1)) - r0) * t5;
}
template<class T> T smith_gtr2(T tt, T a)
{
    if(tt == 0)
        return T(1);
    T root = a * tt;
    return T(2) / (T(1) + std::sqrt(T(1) + root * root));
}
template<class T> T aniso_gtr2(T sph, T cph, T sth, T cth, T ax, T ay)
{
    T A = sq(cph / ax) + sq(sph / ay);
    T RD = sq(sth) * A + sq(cth);
    return T(1) / (PI_T<T>() * ax * ay * sq(RD));
}
template<class T> T smith_aniso(T cp, T sp, T ax, T ay, T tt)
{
    T t = sq(ax * cp) + sq(ay * sp);
    T lambda = T(-0.5) + T(0.5) * std::sqrt(T(1) + t * sq(tt));
    return T(1) / (T(1) + lambda);
}
template<class T> V<T> sample_aniso_gtr2(T ax, T ay, T s0, T s1)
{
    T sp, cp;
    sincos_pi(T(2) * s0, sp, cp);
    T sph = ay * sp;
    T cph = ax * cp;
    T nor = T(1) / std::sqrt(sq(sph) + sq(cph));
    sph *= nor;
    cph *= nor;
    T A = sq(cph / ax) + sq(sph / ay);
    T cth = std::sqrt(A * (T(1) - s1) / ((T(1) - A) * s1 + A));
    T sth = cos2sin(cth);
    return nrm(V<T>(sth * cph, sth * sph, cth));
}
template<class T> T gtr1(T sth, T cth, T a)
{
    return (sq(a) - 1) / (T(2) * PI_T<T>() * std::log(a) * (sq(a * cth) + sq(sth)));
}
template<class T> V<T> sample_gtr1(T a, T s0, T s1)
{
    T cth = std::sqrt((std::pow(a, T(2) - T(2) * s1) - T(1)) / (sq(a) - T(1)));
    T sth = cos2sin(cth);
    T sp, cp;
    sincos_pi(T(2) * s0, sp, cp);
    return nrm(V<T>(sth * cp, sth * sp, cth));
}
template<class T> V<T> sample_vndf(V<T> ve, T ax, T ay, T s0, T s1)
{
    V<T> vh = nrm(V<T>(ax * ve.x, ay * ve.y, ve.z));
    T lensq = vh.x * vh.x + vh.y * vh.y;
    V<T> t1(1, 0, 0);
    if(lensq > T(3e-4))
        t1 = V<T>(-vh.y, vh.x, 0) / std::sqrt(lensq);
    V<T> t2 = cross(vh, t1);
    T r = std::sqrt(s0), sp, cp;
    sincos_pi(T(2) * s1, sp, cp);
    T a1 = r * cp, a2_ = r * sp;
    T s = T(0.5) * (T(1) + vh.z);
    T a2 = (T(1) - s) * std::sqrt(T(1) - a1 * a1) + s * a2_;
    V<T> nh = a1 * t1 + a2 * t2 + std::sqrt(std::max(T(0), T(1) - a1 * a1 - a2 * a2)) * vh;
    return nrm(V<T>(ax * nh.x, ay * nh.y, std::max(T(0), nh.z)));
}

// material record: type, p[0..14]
template<class T>
struct Mat
{
    int type = 0;
    V<T> C;
    // metal
    T ax = 0, ay = 0;
    // disney
    V<T> Ct;
    T metallic = 0, rough = 0, spec = 0, spec_tint = 0, aniso = 0, sheen = 0, sheen_tint = 0, cc = 0, cc_rough = 0,
      trans = 0, trans_rough = 0, ior = 1.5, tax = 0, tay = 0, wd = 0, ws = 0, wc = 0, wt = 0;

    void init(int tp, const float *p)
    {
        type = tp;
        C = V<T>(T(p[0]), T(p[1]), T(p[2]));
        if(tp == 1)
        {
            // MicrofacetReflectionComponentImpl ctor (microfacet_reflection.h:20-33)
            const T r = T(p[3]), an = T(p[4]);
            T aspect = 1;
            if(an > 0)
                aspect = std::sqrt(T(1) - T(0.9) * an);
            ax = std::max(T(0.001), r * r / aspect);
            ay = std::max(T(0.001), r * r * aspect);
        }
        else if(tp == 2)
        {
            // DisneyBSDF ctor (disney.cpp:426-475)
            const T l = lum(C);
            Ct = l > 0 ? C / l : V<T>(T(1));
            metallic = T(p[3]);
            rough = T(p[4]);
            spec = T(p[5]);
            spec_tint = T(p[6]);
            aniso = T(p[7]);
            sheen = T(p[8]);
            sheen_tint = T(p[9]);
            cc = T(p[10]);
            const T gloss = T(p[11]);
            trans = T(p[12]);
            trans_rough = T(p[13]);
            ior = std::max(T(1.01), T(p[14]));
            T aspect = 1;
            if(aniso > 0)
                aspect = std::sqrt(T(1) - T(0.9) * aniso);
            ax = std::max(T(0.001), sq(rough) / aspect);
            ay = std::max(T(0.001), sq(rough) * aspect);
            tax = std::max(T(0.001), sq(trans_rough) / aspect);
            tay = std::max(T(0.001), sq(trans_rough) * aspect);
            cc_rough = std::max(T(0.0001), sq(lerp1(T(0.1), T(0), gloss)));
            const T A = clampv(l * (T(1) - metallic), T(0.3), T(0.7));
            const T B = T(1) - A;
            wd = A * (T(1) - trans);
            wt = A * trans;
            ws = B * T(2) / (T(2) + cc);
            wc = B * cc / (T(2) + cc);
        }
    }

    // ---- metal (microfacet_reflection.h:78-121)
    void metal_ep(V<T> wi, V<T> wo, V<T> &f, T &pdf) const
    {
        if(wi.z <= 0 || wo.z <= 0)
        {
            f = V<T>(0);
            pdf = 0;
            return;
        }
        V<T> wh = nrm(wi + wo);
        T ctd = dot(wi, wh);
        T ph = phi_of(wh);
        T D = aniso_gtr2(std::sin(ph), std::cos(ph), cos2sin(wh.z), wh.z, ax, ay);
        T pi_ = phi_of(wi), po = phi_of(wo);
        T Go = smith_aniso(std::cos(po), std::sin(po), ax, ay, tan_th(wo));
        T Gi = smith_aniso(std::cos(pi_), std::sin(pi_), ax, ay, tan_th(wi));
        f = schlick3(C, ctd) * (D * Gi * Go / std::abs(T(4) * wi.z * wo.z));
        pdf = Go * D / (T(4) * wo.z);
    }

    // ---- disney lobes (disney.cpp:76-422)
    static T om5(T x)
    {
        T t = T(1) - x, t2 = t * t;
        return t2 * t2 * t;
    }
    V<T> d_trans(V<T> wi, V<T> wo) const
    {
        T ci = wi.z, co = wo.z;
        T eta = co > 0 ? ior : T(1) / ior;
        V<T> wh = nrm(wo + eta * wi);
        if(wh.z < 0)
            wh = -wh;
        T ctd = dot(wo, wh);
        T F = diel_fresnel(ior, T(1), ctd);
        T ph = phi_of(wh);
        T D = aniso_gtr2(std::sin(ph), std::cos(ph), cos2sin(wh.z), wh.z, tax, tay);
        T pi_ = phi_of(wi), po = phi_of(wo);
        T G = smith_aniso(std::cos(pi_), std::sin(pi_), tax, tay, tan_th(wi)) *
              smith_aniso(std::cos(po), std::sin(po), tax, tay, tan_th(wo));
        T sdem = ctd + eta * dot(wi, wh);
        T corr = T(1) / eta;
        V<T> sqrtC(std::sqrt(C.x), std::sqrt(C.y), std::sqrt(C.z));
        T val = (T(1) - F) * D * G * eta * eta * dot(wi, wh) * dot(wo, wh) * corr * corr / (ci * co * sdem * sdem);
        T tf = co > 0 ? trans : T(1);
        return (T(1) - metallic) * tf * sqrtC * std::abs(val);
    }
    V<T> d_inner(V<T> wi, V<T> wo) const
    {
        V<T> wh = -nrm(wi + wo);
        T ctd = dot(wo, wh);
        T F = diel_fresnel(ior, T(1), ctd);
        T ph = phi_of(wh);
        T D = aniso_gtr2(std::sin(ph), std::cos(ph), cos2sin(wh.z), wh.z, tax, tay);
        T pi_ = phi_of(wi), po = phi_of(wo);
        T G = smith_aniso(std::cos(pi_), std::sin(pi_), tax, tay, tan_th(wi)) *
              smith_aniso(std::cos(po), std::sin(po), tax, tay, tan_th(wo));
        return trans * C * std::abs(F * D * G / (T(4) * wi.z * wo.z));
    }
    V<T> d_spec(V<T> wi, V<T> wo) const
    {
        T ci = wi.z, co = wo.z;
        V<T> wh = nrm(wi + wo);
        T ctd = dot(wi, wh);
        V<T> Cs = lerp(lerp(V<T>(T(1)), Ct, spec_tint), C, metallic);
        V<T> Fd = Cs * diel_fresnel(ior, T(1), ctd);
        V<T> Fc = schlick3(Cs, ctd);
        V<T> F = lerp(spec * Fd, Fc, metallic);
        T ph = phi_of(wh);
        T D = aniso_gtr2(std::sin(ph), std::cos(ph), cos2sin(wh.z), wh.z, ax, ay);
        T pi_ = phi_of(wi), po = phi_of(wo);
        T G = smith_aniso(std::cos(pi_), std::sin(pi_), ax, ay, tan_th(wi)) *
              smith_aniso(std::cos(po), std::sin(po), ax, ay, tan_th(wo));
        return F * D * G / std::abs(T(4) * ci * co);
    }
    V<T> disney_eval(V<T> wi, V<T> wo) const
    {
        if(std::abs(wi.z) < T(1e-4) || std::abs(wo.z) < T(1e-4))
            return V<T>(0);
        if(wi.z * wo.z < 0)
            return trans == 0 ? V<T>(0) : d_trans(wi, wo);
        if(wi.z < 0 && wo.z < 0)
            return trans == 0 ? V<T>(0) : d_inner(wi, wo);
        if(wi.z <= 0 || wo.z <= 0)
            return V<T>(0);
        T ci = wi.z, co = wo.z;
        V<T> wh = nrm(wi + wo);
        T ctd = dot(wi, wh);
        V<T> diffuse(0), sh(0);
        if(metallic < 1)
        {
            V<T> lam = C / PI_T<T>();
            T fl = om5(ci), fv = om5(co);
            T rr = T(2) * rough * ctd * ctd;
            V<T> retro = C / PI_T<T>() * rr * (fl + fv + fl * fv * (rr - 1));
            diffuse = lam * (T(1) - T(0.5) * fl) * (T(1) - T(0.5) * fv) + retro;
            if(sheen > 0)
                sh = T(4) * sheen * lerp(V<T>(T(1)), Ct, sheen_tint) * om5(ctd);
        }
        V<T> specular = d_spec(wi, wo);
        V<T> clear(0);
        if(cc > 0)
        {
            T D = gtr1(cos2sin(wh.z), wh.z, cc_rough);
            T F = schlick1(T(0.04), ctd);
            T G = smith_gtr2(tan_th(wi), T(0.25)) * smith_gtr2(tan_th(wo), T(0.25));
            T v = cc * D * F * G / std::abs(T(4) * ci * co);
            clear = V<T>(v);
        }
        return (T(1) - metallic) * (T(1) - trans) * (diffuse + sh) + specular + clear;
    }
    T p_trans(V<T> wi, V<T> wo) const
    {
        T eta = wo.z > 0 ? ior : T(1) / ior;
        V<T> wh = nrm(wo + eta * wi);
        if(wh.z < 0)
            wh = -wh;
        if(((wo.z > 0) != (dot(wh, wo) > 0)) || ((wi.z > 0) != (dot(wh, wi) > 0)))
            return 0;
        T sdem = dot(wo, wh) + eta * dot(wi, wh);
        T dd = eta * eta * dot(wi, wh) / (sdem * sdem);
        T ph = phi_of(wh);
        T D = aniso_gtr2(std::sin(ph), std::cos(ph), cos2sin(wh.z), wh.z, tax, tay);
        return std::abs(dot(wi, wh) * D * dd);
    }
    T p_inner(V<T> wi, V<T> wo) const
    {
        V<T> wh = -nrm(wi + wo);
        T ph = phi_of(wh);
        T D = aniso_gtr2(std::sin(ph), std::cos(ph), cos2sin(wh.z), wh.z, tax, tay);
        return std::abs(wh.z * D / (T(4) * dot(wi, wh)));
    }
    T disney_pdf(V<T> wi, V<T> wo) const
    {
        if(std::abs(wi.z) < T(1e-4) || std::abs(wo.z) < T(1e-4))
            return 0;
        if(wo.z < 0)
        {
            if(trans == 0)
                return 0;
            T mF = clampv(diel_fresnel(ior, T(1), wo.z), T(0.1), T(0.9));
            if(wi.z > 0)
                return (T(1) - mF) * p_trans(wi, wo);
            return mF * p_inner(wi, wo);
        }
        if(wi.z < 0)
            return wt * p_trans(wi, wo);
        T diffuse = pdf_hemi_zw(wi);
        V<T> wh = nrm(wi + wo);
        T ph = phi_of(wh);
        T cth = wh.z, sth = cos2sin(cth);
        T ctd = dot(wi, wh);
        T cpo = std::cos(phi_of(wo));
        T spo = cos2sin(cpo);  // the reference uses sqrt(1 - cos^2) here (disney.cpp:335)
        T sD = aniso_gtr2(std::sin(ph), std::cos(ph), sth, cth, ax, ay);
        T ps = smith_aniso(cpo, spo, ax, ay, tan_th(wo)) * sD / (T(4) * wo.z);
        T cD = gtr1(sth, cth, cc_rough);
        T pc = cth * cD / (T(4) * ctd);
        return wd * diffuse + ws * ps + wc * pc;
    }
    V<T> s_trans(V<T> wo, T s0, T s1) const
    {
        V<T> wh = sample_aniso_gtr2(tax, tay, s0, s1);
        if(wh.z <= 0)
            return V<T>(0);
        if((wo.z > 0) != (dot(wh, wo) > 0))
            return V<T>(0);
        T eta = wo.z > 0 ? T(1) / ior : ior;
        V<T> owh = dot(wh, wo) > 0 ? wh : -wh;
        T cti = dot(wo, owh);
        T s2t = eta * eta * (T(1) - cti * cti);
        T c2t = T(1) - s2t;
        if(c2t <= 0)
            return V<T>(0);
        V<T> wi = nrm((eta * cti - std::sqrt(c2t)) * owh - eta * wo);
        if(wi.z * wo.z > 0 || ((wi.z > 0) != (dot(wh, wi) > 0)))
            return V<T>(0);
        return nrm(wi);
    }
    V<T> s_inner(V<T> wo, T s0, T s1) const
    {
        V<T> wh = sample_aniso_gtr2(tax, tay, s0, s1);
        if(wh.z <= 0)
            return V<T>(0);
        V<T> wi = T(2) * dot(wo, wh) * wh - wo;
        if(wi.z > 0)
            return V<T>(0);
        return nrm(wi);
    }
    V<T> s_spec(V<T> wo, T s0, T s1) const
    {
        V<T> wh = sample_vndf(wo, ax, ay, s0, s1);
        if(wh.z <= 0)
            return V<T>(0);
        V<T> wi = T(2) * dot(wo, wh) * wh - wo;
        if(wi.z <= 0)
            return V<T>(0);
        return nrm(wi);
    }
    V<T> s_clear(V<T> wo, T s0, T s1) const
    {
        V<T> wh = sample_gtr1(cc_rough, s0, s1);
        if(wh.z <= 0)
            return V<T>(0);
        V<T> wi = T(2) * dot(wo, wh) * wh - wo;
        if(wi.z <= 0)
            return V<T>(0);
        return nrm(wi);
    }
    CS<T> disney_sample(V<T> wo, T s0, T s1, T s2) const
    {
        CS<T> r;
        if(std::abs(wo.z) < T(1e-4))
            return r;
        V<T> wi;
        if(wo.z < 0)
        {
            if(trans == 0)
                return r;
            T mF = clampv(diel_fresnel(ior, T(1), wo.z), T(0.1), T(0.9));
            wi = s0 >= mF ? s_trans(wo, s1, s2) : s_inner(wo, s1, s2);
        }
        else
        {
            T sel = s0;
            if(sel < wd)
                wi = hemi_zw(s1, s2);
            else
            {
                sel -= wd;
                if(sel < wt)
                    wi = s_trans(wo, s1, s2);
                else
                {
                    sel -= wt;
                    wi = sel < ws ? s_spec(wo, s1, s2) : s_clear(wo, s1, s2);
                }
            }
        }
        if(zero3(wi))
            return r;
        r.dir = wi;
        r.f = disney_eval(wi, wo);
        r.pdf = disney_pdf(wi, wo);
        V<T> v = r.f * (std::abs(wi.z) / r.pdf);
        if(!keep_bad && std::max(std::max(v.x, v.y), v.z) > T(10))
            return CS<T>();
        return r;
    }
    bool keep_bad = false;  // test hook: skip handle_bad_sample to expose the raw sampling density

    // ---- component dispatch (diffuse.cpp:10-60, metal, disney)
    CS<T> sample(V<T> wo, T s0, T s1, T s2) const
    {
        CS<T> r;
        if(type == 0)
        {
            if(wo.z <= 0)
                return r;
            r.dir = hemi_zw(s1, s2);
            r.f = C / PI_T<T>();
            r.pdf = pdf_hemi_zw(r.dir);
            return r;
        }
        if(type == 1)
        {
            if(wo.z > 0)
            {
                V<T> wh = nrm(sample_vndf(wo, ax, ay, s1, s2));
                if(wh.z > 0)
                {
                    V<T> wi = nrm(T(2) * dot(wo, wh) * wh - wo);
                    if(wi.z > 0)
                    {
                        r.dir = wi;
                        metal_ep(wi, wo, r.f, r.pdf);
                    }
                }
            }
            return r;
        }
        return disney_sample(wo, s0, s1, s2);
    }
    V<T> eval(V<T> wi, V<T> wo) const
    {
        if(type == 0)
            return (wi.z <= 0 || wo.z <= 0) ? V<T>(0) : C / PI_T<T>();
        if(type == 1)
        {
            V<T> f;
            T p;
            metal_ep(wi, wo, f, p);
            return f;
        }
        return disney_eval(wi, wo);
    }
    T pdf(V<T> wi, V<T> wo) const
    {
        if(type == 0)
            return (wi.z <= 0 || wo.z <= 0) ? T(0) : pdf_hemi_zw(wi);
        if(type == 1)
        {
            V<T> f;
            T p;
            metal_ep(wi, wo, f, p);
            return p;
        }
        return disney_pdf(wi, wo);
    }
};

} // namespace orc

using namespace orc;

// ------------------------------------------------------------------ scene for the renderer

struct OracleScene
{
    const float *tris;      // 9 floats per flattened world triangle
    const uint32_t *ids;    // (instance, primitive) per flattened triangle
    uint64_t ntri;

    int32_t ninst;
    const float *inst_l2w;  // 12 per instance, rows of the 3x4 local-to-world matrix
    const float *inst_w2l;  // 12 per instance, the reference's stored inverse
    const int32_t *inst_geo, *inst_mat, *inst_light, *inst_inner, *inst_outer;

    int32_t ngeo;
    const uint64_t *geo_offset, *geo_count;
    const float *geo_area_total;
    const float *shade;     // [6][total_geo_tris][4]
    uint64_t total_geo_tris;
    const float *tri_area;  // per geometry triangle
    const float *local_pos; // 9 per geometry triangle: a, b, c (object space)

    int32_t nmat;
    const float *mat;       // 20 per material: type, shadow_terminator, p[16], pad, pad

    int32_t nlight;
    const int32_t *light_inst, *light_geo;
    const float *light_scale, *light_intensity;
    int32_t env_type;
    float env_lower[3], env_upper[3], env_up[3];

    int32_t vacuum_medium;
    float world_diagonal;
    int32_t nmed;
    const float *med;       // 28 floats per medium (layout in medium() below)
    const uint64_t *med_grid_offset;
    const float *grids;

    float eye[3], lbc[3], film_x[3], film_y[3];
    int32_t width, height, spp, min_depth, max_depth;
    float rr_threshold, rr_cont_prob;
    int32_t sampler, filter;
    float filter_radius, filter_alpha;

    int32_t nvol;           // volumes[] in file order
    const float *vol;       // 32 floats per volume (layout at volume() below)
    const uint64_t *vol_off; // 2 per volume: sigma_t grid, albedo grid offsets into grids

    // 2D textures (layouts at OTexImage / OTexInstr / OMatTex below)
    int32_t ntex_img;
    const void *tex_img;
    const float *tex_texels;   // 4 floats per texel
    const void *tex_instr;
    const void *mat_tex;
    const int32_t *mat_texrow; // per material: row of mat_tex or -1
    int32_t env_prog, env_lut_w, env_lut_h;  // env_type 2 (ibl); env_up holds its "up"
};

namespace {

struct Prepared
{
    const OracleScene *S;
    Bvh bvh;
    std::vector<Alias> geo_alias;   // only for light geometries
    Alias filter;
    Sampler::HC hc;
    bool has_media = false;
    // ibl importance table (EnvirLightSampler::preprocess, env_sampler.cpp:83-135)
    std::vector<float> env_probs;
    Alias env_alias;
    Frame<float> env_frame;
};

V3f pt(const float *m, V3f p)
{
    return V3f(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
               m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}
V3f vec(const float *m, V3f v)
{
    return V3f(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
               m[8] * v.x + m[9] * v.y + m[10] * v.z);
}
V3f nor(const float *inv, V3f n)
{
    return V3f(inv[0] * n.x + inv[4] * n.y + inv[8] * n.z, inv[1] * n.x + inv[5] * n.y + inv[9] * n.z,
               inv[2] * n.x + inv[6] * n.y + inv[10] * n.z);
}

// intersection_offset (common/btrc/utils/intersection.cpp:5-37)
V3f ioffset(V3f pos, V3f n)
{
    const float ORIGIN = 1.0f / 32.0f, FS = 1.0f / 65536.0f, IS = 256.0f;
    auto one = [&](float p, float nn) {
        const int of = static_cast<int>(2 * IS * nn);
        int32_t pi;
        std::memcpy(&pi, &p, 4);
        pi += p < 0 ? -of : of;
        float pf;
        std::memcpy(&pf, &pi, 4);
        return std::fabs(p) < ORIGIN ? p + FS * nn : pf;
    };
    return V3f(one(pos.x, n.x), one(pos.y, n.y), one(pos.z, n.z));
}
V3f ioffset_dir(V3f pos, V3f n, V3f d) { return ioffset(pos, dot(n, d) > 0 ? n : -n); }

V3f sky(const OracleScene &S, V3f d)
{
    const V3f up(S.env_up[0], S.env_up[1], S.env_up[2]);
    const float c = dot(up, nrm(d));
    const float s = std::min(1.0f, std::max(0.0f, 0.5f * (c + 1.0f)));
    return V3f(S.env_lower[0], S.env_lower[1], S.env_lower[2]) * (1.0f - s) +
           V3f(S.env_upper[0], S.env_upper[1], S.env_upper[2]) * s;
}

int nlights_total(const OracleScene &S) { return S.nlight + (S.env_type ? 1 : 0); }

// ---- 2D textures: image textures in normalised coordinates with the address modes and
// filters of a CUDA texture object (common/btrc/utils/cuda/texture.cpp:62-102, exact
// bilinear weights), and postfix programs for add / sub / mul / div and uv transforms
// (builtin/btrc/builtin/texture2d/{array2d,math,transform}.cpp)
struct OTexImage
{
    int32_t offset, width, height, filter, au, av, pad0, pad1;
    float border[4];
};
struct OTexInstr
{
    int32_t op, image;   // op: 0 end, 1 const, 2 sample, 3 add, 4 sub, 5 mul, 6 div
    float a[6];
};
struct OMatTex
{
    int32_t prog[16];
    int32_t normal;
    int32_t pad[3];
};

bool otex_index(int i, int n, int mode, int &out)
{
    if(mode == 0)  // wrap
    {
        const int m = i % n;
        out = m < 0 ? m + n : m;
        return true;
    }
    if(mode == 2)  // mirror
    {
        int m = i % (2 * n);
        m = m < 0 ? m + 2 * n : m;
        out = m < n ? m : 2 * n - 1 - m;
        return true;
    }
    if(mode == 3)  // border
    {
        out = i;
        return i >= 0 && i < n;
    }
    out = std::min(std::max(i, 0), n - 1);  // clamp
    return true;
}

V3f otex_fetch(const OracleScene &S, const OTexImage &im, int x, int y)
{
    int ix, iy;
    const bool a = otex_index(x, im.width, im.au, ix), b = otex_index(y, im.height, im.av, iy);
    if(!a || !b)
        return V3f(im.border[0], im.border[1], im.border[2]);
    const float *t = S.tex_texels + (static_cast<int64_t>(im.offset) + static_cast<int64_t>(iy) * im.width + ix) * 4;
    return V3f(t[0], t[1], t[2]);
}

float otex_coord(float u, int mode)
{
    if(mode == 0)
        return u - std::floor(u);
    if(mode == 2)
    {
        const float f = std::floor(u), r = u - f;
        return (static_cast<int>(f) & 1) ? 1.0f - r : r;
    }
    return u;
}

V3f otex_sample(const OracleScene &S, const OTexImage &im, float u, float v)
{
    u = otex_coord(u, im.au);
    v = otex_coord(v, im.av);
    if(!(u == u) || !(v == v))
        return V3f(0.0f);
    auto lim = [](float x) { return std::min(std::max(x, -1.0e9f), 1.0e9f); };
    if(im.filter == 0)
        return otex_fetch(S, im, static_cast<int>(std::floor(lim(u * im.width))),
                          static_cast<int>(std::floor(lim(v * im.height))));
    const float xb = lim(u * im.width - 0.5f), yb = lim(v * im.height - 0.5f);
    const float fx = std::floor(xb), fy = std::floor(yb), ax = xb - fx, ay = yb - fy;
    const int x0 = static_cast<int>(fx), y0 = static_cast<int>(fy);
    const V3f t00 = otex_fetch(S, im, x0, y0), t10 = otex_fetch(S, im, x0 + 1, y0);
    const V3f t01 = otex_fetch(S, im, x0, y0 + 1), t11 = otex_fetch(S, im, x0 + 1, y0 + 1);
    return (t00 * (1.0f - ax) + t10 * ax) * (1.0f - ay) + (t01 * (1.0f - ax) + t11 * ax) * ay;
}

V3f otex_eval(const OracleScene &S, int prog, float u, float v)
{
    const OTexInstr *code = static_cast<const OTexInstr *>(S.tex_instr);
    const OTexImage *imgs = static_cast<const OTexImage *>(S.tex_img);
    std::vector<V3f> st;
    for(int k = prog;; ++k)
    {
        const OTexInstr &ins = code[k];
        if(ins.op == 1)
            st.push_back(V3f(ins.a[0], ins.a[1], ins.a[2]));
        else if(ins.op == 2)
            st.push_back(otex_sample(S, imgs[ins.image], ins.a[0] * u + ins.a[1] * v + ins.a[2],
                                     ins.a[3] * u + ins.a[4] * v + ins.a[5]));
        else if(ins.op >= 3 && ins.op <= 6)
        {
            const V3f r = st.back();
            st.pop_back();
            V3f &l = st.back();
            l = ins.op == 3 ? l + r : ins.op == 4 ? l - r : ins.op == 5 ? l * r : l / r;
        }
        else
            return st.empty() ? V3f(0.0f) : st.back();
    }
}

// ---- ibl (builtin/btrc/builtin/light/ibl.cpp, env_sampler.cpp)
float local_phi(V3f d)
{
    float phi = 0.0f;
    if(d.x != 0 || d.y != 0)
    {
        phi = std::atan2(d.y, d.x);
        if(phi < 0)
            phi += 2 * PIf;
    }
    return phi;
}

V3f ibl_eval_local(const OracleScene &S, V3f d)
{
    const float theta = std::acos(std::min(std::max(d.z, -1.0f), 1.0f));
    const float u = std::min(std::max(1 / (2 * PIf) * local_phi(d), 0.0f), 1.0f);
    const float v = std::min(std::max(1 / PIf * theta, 0.0f), 1.0f);
    return otex_eval(S, S.env_prog, u, v);
}

V3f env_le(const Prepared &P, V3f d)
{
    if(P.S->env_type == 2)
        return ibl_eval_local(*P.S, nrm(P.env_frame.g2l(d)));
    return sky(*P.S, d);
}

// pdf_li of the environment light; EnvirLightSampler::pdf (env_sampler.cpp:165-187) for ibl
float env_pdf(const Prepared &P, V3f d)
{
    const OracleScene &S = *P.S;
    if(S.env_type != 2)
        return 1.0f / (4.0f * PIf);
    const V3f dir = nrm(P.env_frame.g2l(d));
    const float theta = std::acos(std::min(std::max(dir.z, -1.0f), 1.0f));
    const float u = local_phi(dir) / (2 * PIf), v = theta / PIf;
    const int w = S.env_lut_w, h = S.env_lut_h;
    const int tx = std::min(std::max(static_cast<int>(std::floor(u * w)), 0), w - 1);
    const int ty = std::min(std::max(static_cast<int>(std::floor(v * h)), 0), h - 1);
    const float u0 = static_cast<float>(tx) / w, u1 = static_cast<float>(tx + 1) / w;
    const float v0 = static_cast<float>(ty) / h, v1 = static_cast<float>(ty + 1) / h;
    return P.env_probs[ty * w + tx] * (1.0f / std::fabs(2 * PIf * (u1 - u0) * (cos_pi(v1) - cos_pi(v0))));
}

void build_env_table(Prepared &P)
{
    const OracleScene &S = *P.S;
    const int w = S.env_lut_w, h = S.env_lut_h;
    std::vector<float> lum(static_cast<size_t>(w) * h), area(lum.size());
    for(int yi = 0; yi < h; ++yi)
        for(int xi = 0; xi < w; ++xi)
        {
            const float x0 = static_cast<float>(xi) / w, x1 = static_cast<float>(xi + 1) / w;
            const float y0 = static_cast<float>(yi) / h, y1 = static_cast<float>(yi + 1) / h;
            float sum = 0;
            for(uint32_t i = 0; i < 256; ++i)
            {
                // Hammersley point (i / 256, radical inverse of i), spread over 1.2x the tile
                uint32_t b = (i << 16u) | (i >> 16u);
                b = ((b & 0x55555555u) << 1u) | ((b & 0xAAAAAAAAu) >> 1u);
                b = ((b & 0x33333333u) << 2u) | ((b & 0xCCCCCCCCu) >> 2u);
                b = ((b & 0x0F0F0F0Fu) << 4u) | ((b & 0xF0F0F0F0u) >> 4u);
                b = ((b & 0x00FF00FFu) << 8u) | ((b & 0xFF00FF00u) >> 8u);
                const float sx = 1.2f * (static_cast<float>(i) / 256) - 0.1f;
                const float sy = 1.2f * (b * 2.3283064365386963e-10f) - 0.1f;
                const V3f c = otex_eval(S, S.env_prog, x0 + (x1 - x0) * sx, y0 + (y1 - y0) * sy);
                sum += 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z;
            }
            lum[yi * w + xi] = sum / 256;
            area[yi * w + xi] = std::fabs(2 * PIf * (x1 - x0) * (std::cos(PIf * y1) - std::cos(PIf * y0)));
        }
    float la = 0, as = 0;
    for(size_t i = 0; i < lum.size(); ++i)
    {
        la += lum[i] * area[i];
        as += area[i];
    }
    const float avg = la / as;
    float total = 0;
    for(size_t i = 0; i < lum.size(); ++i)
    {
        lum[i] = std::max(0.0f, area[i] * (lum[i] - avg));
        total += lum[i];
    }
    if(total > 1e-3f)
        for(float &v : lum)
            v *= 1 / total;
    P.env_probs = lum;
    P.env_alias.init(lum);
}

struct ShadeFrame
{
    Frame<float> g, s;
    bool black(V3f w) const { return g.upper(w) != s.upper(w); }
    ShadeFrame flip(V3f wo) const
    {
        ShadeFrame f;
        f.g = g;
        f.s = black(wo) ? g : s;
        return f;
    }
    float corr(V3f wi) const
    {
        const float down = std::fabs(dot(g.z, wi));
        return down > 1e-4f ? std::fabs(dot(s.z, wi)) / down : 1.0f;
    }
    float term(V3f wi) const
    {
        const float a = dot(g.z, wi), b = dot(s.z, wi), c = dot(g.z, s.z);
        const float t = std::min(1.0f, std::max(0.0f, a / (b * c)));
        return -t * t * t + t * t + t;
    }
};

// ---- participating media (builtin/btrc/builtin/medium/{hetergeneous,homogeneous}.cpp,
// core/btrc/core/medium.cpp, common/btrc/utils/henyey_greenstein.h)
// medium record: [0] type (0 vacuum, 1 homogeneous, 2 heterogeneous), [1] priority,
// [2..4] grid resolution, [5] unused (offsets in med_grid_offset), [6] sigma_max, [7] g, [8] homogeneous sigma_t,
// [9..11] albedo, [12..23] world-to-local 3x4 rows
struct Med
{
    int type;
    int rx, ry, rz;
    uint64_t off;
    float sigma_max, g, sigma_t;
    V3f albedo;
    const float *w2l;
};

Med medium(const OracleScene &S, int id)
{
    const float *r = S.med + id * 28;
    Med m;
    m.type = static_cast<int>(r[0]);
    m.rx = static_cast<int>(r[2]);
    m.ry = static_cast<int>(r[3]);
    m.rz = static_cast<int>(r[4]);
    m.off = S.med_grid_offset[id];
    m.sigma_max = r[6];
    m.g = r[7];
    m.sigma_t = r[8];
    m.albedo = V3f(r[9], r[10], r[11]);
    m.w2l = r + 12;
    return m;
}

float grid_at(const OracleScene &S, const Med &m, V3f uvw)
{
    const float fx = uvw.x * m.rx - 0.5f, fy = uvw.y * m.ry - 0.5f, fz = uvw.z * m.rz - 0.5f;
    const float flx = std::floor(fx), fly = std::floor(fy), flz = std::floor(fz);
    const float tx = fx - flx, ty = fy - fly, tz = fz - flz;
    auto cl = [](int v, int n) { return std::min(std::max(v, 0), n - 1); };
    const int x0 = cl(int(flx), m.rx), x1 = cl(int(flx) + 1, m.rx);
    const int y0 = cl(int(fly), m.ry), y1 = cl(int(fly) + 1, m.ry);
    const int z0 = cl(int(flz), m.rz), z1 = cl(int(flz) + 1, m.rz);
    const float *g = S.grids + m.off;
    auto at = [&](int x, int y, int z) { return g[(static_cast<size_t>(z) * m.ry + y) * m.rx + x]; };
    const float c00 = at(x0, y0, z0) + (at(x1, y0, z0) - at(x0, y0, z0)) * tx;
    const float c10 = at(x0, y1, z0) + (at(x1, y1, z0) - at(x0, y1, z0)) * tx;
    const float c01 = at(x0, y0, z1) + (at(x1, y0, z1) - at(x0, y0, z1)) * tx;
    const float c11 = at(x0, y1, z1) + (at(x1, y1, z1) - at(x0, y1, z1)) * tx;
    const float c0 = c00 + (c10 - c00) * ty, c1 = c01 + (c11 - c01) * ty;
    return c0 + (c1 - c0) * tz;
}

// ---- volume primitives: VolumePrimitiveMedium (core/btrc/core/volume.cpp:112-197),
// volume::BVH queries (core/btrc/core/volume/bvh.cpp:127-327) answered by brute force over
// all boxes (the nearest crossing and the containing set do not depend on the tree), and
// volume::Aggregate tracking (core/btrc/core/volume/aggregate.cpp:131-252).
// volume record: [0..2] o, [3..5] x, [6..8] y, [9..11] z, [12] constant sigma_t,
// [13] max sigma_t, [14..16] sigma grid res, [17..19] albedo grid res, [20] albedo
// channels (1 or 3), [21..23] constant albedo, [24] sigma is a grid, [25] albedo is a grid
struct Vol
{
    V3f o, x, y, z, xd, yd, zd;
    float xi, yi, zi;
    float sigma_const, sigma_max;
    int sres[3], ares[3], ach;
    V3f albedo_const;
    bool sgrid, agrid;
    uint64_t soff, aoff;
};

Vol volume(const OracleScene &S, int k)
{
    const float *r = S.vol + k * 32;
    Vol v;
    v.o = V3f(r[0], r[1], r[2]);
    v.x = V3f(r[3], r[4], r[5]);
    v.y = V3f(r[6], r[7], r[8]);
    v.z = V3f(r[9], r[10], r[11]);
    v.xi = 1.0f / dot(v.x, v.x);
    v.yi = 1.0f / dot(v.y, v.y);
    v.zi = 1.0f / dot(v.z, v.z);
    v.xd = v.x / dot(v.x, v.x);
    v.yd = v.y / dot(v.y, v.y);
    v.zd = v.z / dot(v.z, v.z);
    v.sigma_const = r[12];
    v.sigma_max = r[13];
    for(int i = 0; i < 3; ++i)
    {
        v.sres[i] = static_cast<int>(r[14 + i]);
        v.ares[i] = static_cast<int>(r[17 + i]);
    }
    v.ach = static_cast<int>(r[20]);
    v.albedo_const = V3f(r[21], r[22], r[23]);
    v.sgrid = r[24] != 0;
    v.agrid = r[25] != 0;
    v.soff = S.vol_off[k * 2];
    v.aoff = S.vol_off[k * 2 + 1];
    return v;
}

float grid_tri(const float *g, int rx, int ry, int rz, int nch, int c, V3f uvw)
{
    const float fx = uvw.x * rx - 0.5f, fy = uvw.y * ry - 0.5f, fz = uvw.z * rz - 0.5f;
    const float flx = std::floor(fx), fly = std::floor(fy), flz = std::floor(fz);
    const float tx = fx - flx, ty = fy - fly, tz = fz - flz;
    auto cl = [](int v, int n) { return std::min(std::max(v, 0), n - 1); };
    const int x0 = cl(int(flx), rx), x1 = cl(int(flx) + 1, rx);
    const int y0 = cl(int(fly), ry), y1 = cl(int(fly) + 1, ry);
    const int z0 = cl(int(flz), rz), z1 = cl(int(flz) + 1, rz);
    auto at = [&](int x, int y, int z) { return g[((static_cast<size_t>(z) * ry + y) * rx + x) * nch + c]; };
    const float c00 = at(x0, y0, z0) + (at(x1, y0, z0) - at(x0, y0, z0)) * tx;
    const float c10 = at(x0, y1, z0) + (at(x1, y1, z0) - at(x0, y1, z0)) * tx;
    const float c01 = at(x0, y0, z1) + (at(x1, y0, z1) - at(x0, y0, z1)) * tx;
    const float c11 = at(x0, y1, z1) + (at(x1, y1, z1) - at(x0, y1, z1)) * tx;
    const float c0 = c00 + (c10 - c00) * ty, c1 = c01 + (c11 - c01) * ty;
    return c0 + (c1 - c0) * tz;
}

V3f vol_uvw(const Vol &v, V3f p)
{
    const V3f op = p - v.o;
    return V3f(dot(op, v.x) * v.xi, dot(op, v.y) * v.yi, dot(op, v.z) * v.zi);
}

float vol_sigma(const OracleScene &S, const Vol &v, V3f uvw)
{
    if(!v.sgrid)
        return v.sigma_const;
    return grid_tri(S.grids + v.soff, v.sres[0], v.sres[1], v.sres[2], 1, 0, uvw);
}

// a one-channel array albedo reads back as (v, 0, 0)
V3f vol_albedo(const OracleScene &S, const Vol &v, V3f uvw)
{
    if(!v.agrid)
        return v.albedo_const;
    const float *g = S.grids + v.aoff;
    if(v.ach == 1)
        return V3f(grid_tri(g, v.ares[0], v.ares[1], v.ares[2], 1, 0, uvw), 0.0f, 0.0f);
    return V3f(grid_tri(g, v.ares[0], v.ares[1], v.ares[2], 3, 0, uvw),
               grid_tri(g, v.ares[0], v.ares[1], v.ares[2], 3, 1, uvw),
               grid_tri(g, v.ares[0], v.ares[1], v.ares[2], 3, 2, uvw));
}

float vol_crossing(const Vol &v, V3f p, V3f d)
{
    const V3f op = p - v.o;
    float t0 = 0.0f, t1 = 1.0f;
    const V3f ax[3] = { v.xd, v.yd, v.zd };
    for(int a = 0; a < 3; ++a)
    {
        const float opd = dot(op, ax[a]), dd = dot(d, ax[a]);
        const float nd = (0.0f - opd) / dd, fd = (1.0f - opd) / dd;
        t0 = std::fmax(t0, std::fmin(nd, fd));
        t1 = std::fmin(t1, std::fmax(nd, fd));
    }
    if(t0 > t1)
        return -1.0f;
    if(t0 > 0)
        return t0;
    if(t1 < 1.0f)
        return t1;
    return -1.0f;
}

bool vol_next_boundary(const OracleScene &S, V3f a, V3f b, V3f &out)
{
    const V3f dir = b - a;
    float best = std::numeric_limits<float>::max();
    for(int k = 0; k < S.nvol; ++k)
    {
        const float t = vol_crossing(volume(S, k), a, dir);
        if(t >= 0.0f)
            best = std::fmin(best, t);
    }
    if(best > 10.0f)
        return false;
    out = a * (1.0f - best) + b * best;
    return true;
}

// the (at most 4) lowest-id volumes containing p
int vol_overlap(const OracleScene &S, V3f p, int *ids)
{
    int n = 0;
    for(int k = 0; k < S.nvol && n < 4; ++k)
    {
        const Vol v = volume(S, k);
        const V3f op = p - v.o;
        const float u = dot(op, v.xd), w = dot(op, v.yd), x = dot(op, v.zd);
        if(0.0f <= u && u <= 1.0f && 0.0f <= w && w <= 1.0f && 0.0f <= x && x <= 1.0f)
            ids[n++] = k;
    }
    return n;
}

float overlap_inv_max(const OracleScene &S, const int *ids, int n)
{
    float m = 0.0f;
    for(int k = 0; k < n; ++k)
        m += volume(S, ids[k]).sigma_max;
    return 1.0f / std::max(m, 0.01f);
}

template<class Smp>
bool vol_sample_overlap(const OracleScene &S, const int *ids, int n, V3f a, V3f b, Smp &smp, V3f &pos, V3f &color)
{
    const float inv = overlap_inv_max(S, ids, n);
    Vol vs[4];
    V3f ua[4], ub[4];
    for(int k = 0; k < n; ++k)
    {
        vs[k] = volume(S, ids[k]);
        ua[k] = vol_uvw(vs[k], a);
        ub[k] = vol_uvw(vs[k], b);
    }
    const float t_max = len(b - a);
    float t = 0.0f;
    for(int it = 0; it < (1 << 20); ++it)
    {
        t += -std::log(1.0f - smp.get1d()) * inv;
        if(t >= t_max)
            return false;
        const float tf = t / t_max;
        float dens[4], sum = 0.0f;
        V3f uvw[4];
        for(int k = 0; k < n; ++k)
        {
            uvw[k] = ua[k] * (1.0f - tf) + ub[k] * tf;
            dens[k] = vol_sigma(S, vs[k], uvw[k]);
            sum += dens[k];
        }
        if(smp.get1d() < sum * inv)
        {
            pos = a * (1.0f - tf) + b * tf;
            V3f alb(0.0f);
            for(int k = 0; k < n; ++k)
                alb = alb + (dens[k] / sum) * vol_albedo(S, vs[k], uvw[k]);
            color = alb;
            return true;
        }
    }
    return false;
}

template<class Smp>
float vol_tr_overlap(const OracleScene &S, const int *ids, int n, V3f a, V3f b, Smp &smp)
{
    const float inv = overlap_inv_max(S, ids, n);
    Vol vs[4];
    V3f ua[4], ub[4];
    for(int k = 0; k < n; ++k)
    {
        vs[k] = volume(S, ids[k]);
        ua[k] = vol_uvw(vs[k], a);
        ub[k] = vol_uvw(vs[k], b);
    }
    const float t_max = len(b - a);
    float r = 1.0f, t = 0.0f;
    for(int it = 0; it < (1 << 20); ++it)
    {
        t += -std::log(1.0f - smp.get1d()) * inv;
        if(t >= t_max)
            break;
        const float tf = t / t_max;
        float sum = 0.0f;
        for(int k = 0; k < n; ++k)
            sum += vol_sigma(S, vs[k], ua[k] * (1.0f - tf) + ub[k] * tf);
        r *= 1.0f - sum * inv;
    }
    return r;
}

template<class Smp>
bool volumes_sample(const OracleScene &S, V3f a, V3f b, Smp &smp, V3f &pos, V3f &color)
{
    V3f o = a;
    const V3f d = nrm(b - a);
    for(int seg = 0; seg < (1 << 16); ++seg)
    {
        if(dot(b - o, d) <= 0.0f || dot(b - o, b - o) < 0.00001f)
            return false;
        V3f inct;
        if(!vol_next_boundary(S, o, b, inct))
            inct = b;
        int ids[4];
        const int n = vol_overlap(S, 0.5f * (o + inct), ids);
        if(n != 0 && vol_sample_overlap(S, ids, n, o, inct, smp, pos, color))
            return true;
        o = inct + 0.001f * d;
    }
    return false;
}

template<class Smp>
float volumes_tr(const OracleScene &S, V3f a, V3f b, Smp &smp)
{
    float r = 1.0f;
    V3f o = a;
    const V3f d = nrm(b - a);
    for(int seg = 0; seg < (1 << 16); ++seg)
    {
        if(dot(b - o, d) <= 0.0f || dot(b - o, b - o) < 0.0001f)
            break;
        V3f inct;
        if(!vol_next_boundary(S, o, b, inct))
            inct = b;
        int ids[4];
        const int n = vol_overlap(S, 0.5f * (o + inct), ids);
        if(n != 0)
            r *= vol_tr_overlap(S, ids, n, o, inct, smp);
        o = inct + 0.001f * d;
    }
    return r;
}

// medium sampling; color / g are the phase function's (the medium's albedo and HG g)
template<class Smp>
bool medium_sample(const OracleScene &S, const Med &m, V3f a, V3f b, Smp &smp, V3f &pos, V3f &color, float &g)
{
    if(m.type == 0)
        return false;
    if(m.type == 3)
    {
        g = 0.0f;
        return volumes_sample(S, a, b, smp, pos, color);
    }
    color = m.albedo;
    g = m.g;
    const float t_max = len(b - a);
    if(m.type == 1)
    {
        const float st = -std::log(1.0f - smp.get1d()) / m.sigma_t;
        if(st < t_max)
        {
            pos = a + nrm(b - a) * st;
            return true;
        }
        return false;
    }
    const float inv = 1.0f / m.sigma_max;
    const V3f la = V3f(0.5f) + 0.5f * pt(m.w2l, a), lb = V3f(0.5f) + 0.5f * pt(m.w2l, b);
    const V3f ls = (lb - la) / t_max, ws = (b - a) / t_max;
    float t = 0;
    for(int it = 0; it < (1 << 20); ++it)
    {
        t += -std::log(1.0f - smp.get1d()) * inv;
        if(t >= t_max)
            return false;
        const float dens = grid_at(S, m, la + t * ls);
        if(smp.get1d() < dens * inv)
        {
            pos = a + t * ws;
            return true;
        }
    }
    return false;
}

template<class Smp>
V3f medium_tr(const OracleScene &S, const Med &m, V3f a, V3f b, Smp &smp)
{
    if(m.type == 0)
        return V3f(1.0f);
    if(m.type == 3)
        return V3f(volumes_tr(S, a, b, smp));
    const float t_max = len(b - a);
    if(m.type == 1)
    {
        const V3f sa = m.sigma_t * (V3f(1.0f) - m.albedo);
        return V3f(std::exp(-t_max * sa.x), std::exp(-t_max * sa.y), std::exp(-t_max * sa.z));
    }
    const float inv = 1.0f / m.sigma_max;
    const V3f la = V3f(0.5f) + 0.5f * pt(m.w2l, a), lb = V3f(0.5f) + 0.5f * pt(m.w2l, b);
    const V3f ls = (lb - la) / t_max;
    float r = 1.0f, t = 0;
    for(int it = 0; it < (1 << 20); ++it)
    {
        t += -std::log(1.0f - smp.get1d()) * inv;
        if(t >= t_max)
            break;
        r *= 1.0f - grid_at(S, m, la + t * ls) * inv;
    }
    return V3f(r);
}

float hg(float g, float u)
{
    const float g2 = g * g;
    const float dem = 1.0f + g2 - 2.0f * (g * u);
    return (1.0f - g2) / (4.0f * PIf * dem * std::sqrt(dem));
}

struct PcgSmp
{
    Pcg p;
    float get1d() { return p.uniform(); }
};

void splat(double *film, int w, uint32_t px, uint32_t py, V3f v)
{
    if(!std::isfinite(v.x) || !std::isfinite(v.y) || !std::isfinite(v.z))
        return;
    double *p = film + (static_cast<size_t>(py) * w + px) * 4;
    p[0] += v.x;
    p[1] += v.y;
    p[2] += v.z;
}

// One camera path with the wavefront integrator's semantics, stage by stage as
// WavefrontPathTracer::render runs them per bounce: trace -> medium -> shade -> shadow
// (generate.cpp:33-87, medium.cpp:28-249, shade.cpp:29-235, shadow.cpp:39-76,
// helper.cpp:9-207).
struct LightSample
{
    bool ok = false;
    V3f o, d, li;
    float t1 = 0, pdf = 0;
};

LightSample sample_light(const Prepared &P, V3f ref, V3f ref_nor, bool offset_origin, Sampler &smp)
{
    const OracleScene &S = *P.S;
    LightSample r;
    float s0, s1, s2;
    smp.get3d(s0, s1, s2);
    const float sel = smp.get1d();
    const int NL = nlights_total(S);
    if(NL == 0)
        return r;
    const int li = std::min(static_cast<int>(sel * static_cast<float>(NL)), NL - 1);
    const float spdf = 1.0f / static_cast<float>(NL);
    if(li < S.nlight)
    {
        // MeshLight::sample_li_inline (builtin/btrc/builtin/light/mesh_light.cpp:31-58)
        const int lg = S.light_geo[li], linst = S.light_inst[li];
        const uint32_t prim = P.geo_alias[lg].sample(s0);
        const float tq = std::sqrt(s1);
        const float u = 1.0f - tq, v = tq * s2;
        const float *lp = S.local_pos + (S.geo_offset[lg] + prim) * 9;
        const V3f a(lp[0], lp[1], lp[2]), b(lp[3], lp[4], lp[5]), c(lp[6], lp[7], lp[8]);
        const V3f lpos = a + (b - a) * u + (c - a) * v;
        const float *ez = S.shade + (2 * S.total_geo_tris + S.geo_offset[lg] + prim) * 4;
        const V3f spos = pt(S.inst_l2w + linst * 12, lpos);
        const V3f snor = nrm(nor(S.inst_w2l + linst * 12, nrm(V3f(ez[0], ez[1], ez[2]))));
        const V3f p2r = ref - spos;
        const float d2 = dot(p2r, p2r);
        const float sc = S.light_scale[li];
        const float pdf_sa = 1.0f / (sc * sc) * (1.0f / S.geo_area_total[lg]) * d2 / std::fabs(dot(snor, nrm(p2r)));
        const V3f I(S.light_intensity[li * 3], S.light_intensity[li * 3 + 1], S.light_intensity[li * 3 + 2]);
        r.li = dot(p2r, snor) > 0 ? I : V3f(0.0f);
        const V3f diff = spos - ref;
        const V3f dstp = ioffset_dir(spos, snor, -diff);
        r.o = offset_origin ? ioffset_dir(ref, ref_nor, diff) : ref;
        r.d = dstp - r.o;
        r.t1 = 1.0f;
        r.pdf = spdf * pdf_sa;
    }
    else if(S.env_type == 2)
    {
        // IBL::sample_li_inline (ibl.cpp:31-42), EnvirLightSampler::sample (env_sampler.cpp:137-163)
        const int w = S.env_lut_w, h = S.env_lut_h;
        const uint32_t tile = P.env_alias.sample(s0);
        const int ty = static_cast<int>(tile) / w, tx = static_cast<int>(tile) % w;
        const float u0 = static_cast<float>(tx) / w, u1 = static_cast<float>(tx + 1) / w;
        const float v0 = static_cast<float>(ty) / h, v1 = static_cast<float>(ty + 1) / h;
        float cv0 = cos_pi(v0), cv1 = cos_pi(v1);
        if(cv0 > cv1)
            std::swap(cv0, cv1);
        const float ct = cv0 + s2 * (cv1 - cv0);
        const float st = std::sqrt(std::max(0.0f, 1.0f - ct * ct));
        float sp, cp;
        sincos_pi(2.0f * (u0 + (u1 - u0) * s1), sp, cp);
        const V3f local(st * cp, st * sp, ct);
        const V3f dir = P.env_frame.l2g(local);
        r.o = offset_origin ? ioffset_dir(ref, ref_nor, dir) : ref;
        r.d = dir;
        r.t1 = FMAX;
        r.li = ibl_eval_local(S, local);
        r.pdf = spdf * (P.env_probs[tile] * (1.0f / (2 * PIf * (u1 - u0) * (cv1 - cv0))));
    }
    else
    {
        const float z = 1.0f - (s0 + s0);
        const float rr = std::sqrt(std::max(0.0f, 1.0f - z * z));
        float sp, cp;
        sincos_pi(2.0f * s1, sp, cp);
        const V3f dir(rr * cp, rr * sp, z);
        r.o = offset_origin ? ioffset_dir(ref, ref_nor, dir) : ref;
        r.d = dir;
        r.t1 = FMAX;
        r.li = sky(S, dir);
        r.pdf = spdf * (1.0f / (4.0f * PIf));
    }
    r.ok = true;
    return r;
}

bool russian_roulette(const OracleScene &S, V3f &beta, int depth, Sampler &smp)
{
    if(depth < S.min_depth)
        return false;
    if(depth >= S.max_depth)
        return true;
    const float sam = smp.get1d();
    if(lum(beta) < S.rr_threshold)
    {
        if(sam > S.rr_cont_prob)
            return true;
        beta = beta / S.rr_cont_prob;
    }
    return false;
}

struct Shadow
{
    bool ok = false;
    V3f o, d, beta;
    float t1 = 0;
    int medium = 0;
    uint64_t seed = 0;  // seed of the PCG stream its medium transmittance draws from
};

// Shadow-ray transmittance stream (the GPU kernels' rule, not the reference's one stream
// per shadow slot of W/soa_buffer.cpp:86-96): PCG seeded by a hash of the path's sampler
// state at the start of the emitting stage (1 medium scattering, 2 surface vertex).
inline uint64_t shadow_stream_seed(uint64_t a, uint64_t b, uint64_t stage)
{
    return mix_bits(a ^ mix_bits(b + stage));
}

void trace_path(const Prepared &P, uint64_t g, double *film, double *aov = nullptr)
{
    const OracleScene &S = *P.S;
    const uint64_t pixels = static_cast<uint64_t>(S.width) * S.height;
    const uint64_t pixel = g % pixels, sample = g / pixels;
    const uint32_t px = static_cast<uint32_t>(pixel % S.width), py = static_cast<uint32_t>(pixel / S.width);
    Sampler smp;
    smp.init(S.sampler, P.hc, px, py, static_cast<uint32_t>(sample));
    float fx, fy;
    if(S.filter == 1)
    {
        const uint32_t cell = P.filter.sample(smp.get1d());
        const uint32_t gy = cell / 256, gx = cell % 256;
        const float r = S.filter_radius;
        const float x0 = -r + 2 * r / 256 * static_cast<float>(gx), x1 = -r + 2 * r / 256 * static_cast<float>(gx + 1);
        const float y0 = -r + 2 * r / 256 * static_cast<float>(gy), y1 = -r + 2 * r / 256 * static_cast<float>(gy + 1);
        fx = lerp1(x0, x1, smp.get1d());
        fy = lerp1(y0, y1, smp.get1d());
    }
    else
    {
        fx = smp.get1d() - 0.5f;
        fy = smp.get1d() - 0.5f;
    }
    const float film_x = (static_cast<float>(px) + 0.5f + fx) / static_cast<float>(S.width);
    const float film_y = (static_cast<float>(py) + 0.5f + fy) / static_cast<float>(S.height);
    (void)smp.get1d();
    const V3f eye(S.eye[0], S.eye[1], S.eye[2]);
    const V3f dst = V3f(S.lbc[0], S.lbc[1], S.lbc[2]) + film_x * V3f(S.film_x[0], S.film_x[1], S.film_x[2]) +
                    film_y * V3f(S.film_y[0], S.film_y[1], S.film_y[2]);
    V3f o = eye, d = nrm(dst - eye);
    float t1 = FMAX;
    int ray_medium = S.vacuum_medium;
    film[(static_cast<size_t>(py) * S.width + px) * 4 + 3] += 1.0;

    V3f beta(1.0f), rad(0.0f), beta_le(1.0f);
    float bsdf_pdf = -1.0f;
    int depth = 0;
    const int NL = nlights_total(S);

    for(;;)
    {
        float od[3] = { o.x, o.y, o.z }, dd[3] = { d.x, d.y, d.z };
        const Bvh::Hit h = P.bvh.closest(od, dd, t1);
        bool alive = false;  // a next state was emitted this bounce
        V3f n_o, n_d, n_beta, n_beta_le;
        float n_pdf = 0;
        int n_medium = 0;
        Shadow sh;

        // ---------------- medium stage (medium.cpp:28-164)
        bool scattered = false;
        if(P.has_media)
        {
            int medium_id;
            V3f end;
            if(h.hit)
            {
                const int inst = static_cast<int>(h.inst);
                const int geo = S.inst_geo[inst];
                const float *ez = S.shade + (2 * S.total_geo_tris + S.geo_offset[geo] + h.prim) * 4;
                const V3f n = nor(S.inst_w2l + inst * 12, V3f(ez[0], ez[1], ez[2]));
                const int im = dot(d, n) < 0 ? S.inst_outer[inst] : S.inst_inner[inst];
                medium_id = std::min(im, ray_medium);
                end = ioffset_dir(o + h.t * d, n, -d);
            }
            else
            {
                medium_id = S.vacuum_medium;
                end = o + nrm(d) * S.world_diagonal;
            }
            ray_medium = medium_id;
            const Med m = medium(S, medium_id);
            if(m.type != 0)
            {
                const uint64_t stage_a = smp.word_a(), stage_b = smp.word_b();
                V3f spos, pcolor;
                float pg = 0.0f;
                const bool sc = medium_sample(S, m, o, end, smp, spos, pcolor, pg);
                const V3f tr = medium_tr(S, m, o, end, smp);
                beta_le = beta_le * tr;
                if(sc)
                {
                    scattered = true;
                    if(russian_roulette(S, beta, depth, smp))
                        splat(film, S.width, px, py, rad);
                    else
                    {
                        LightSample ls = sample_light(P, spos, V3f(0, 0, 1), false, smp);
                        if(ls.ok)
                        {
                            const float u = -dot(nrm(ls.d), nrm(-d));
                            const float ph = hg(pg, u);
                            ls.li = ls.li * beta * (pcolor * ph) / (ph + ls.pdf);
                        }
                        // HenyeyGreensteinPhaseShader::sample (core/btrc/core/medium.cpp:32-64)
                        float a0, a1, a2;
                        smp.get3d(a0, a1, a2);
                        const float ss = a0 + a0 - 1;
                        float u;
                        if(std::fabs(pg) < 0.001f)
                            u = ss;
                        else
                        {
                            const float g2 = pg * pg;
                            u = (1.0f + g2 - sq((1.0f - g2) / (1.0f + pg * ss))) / (pg + pg);
                        }
                        const float ct = -u, st = cos2sin(ct);
                        float sp, cp;
                        sincos_pi(2.0f * a1, sp, cp);
                        const V3f lwi(st * sp, st * cp, ct);
                        const float pv = hg(pg, u);
                        const V3f phase = pcolor * pv;
                        const V3f nd = Frame<float>::from_z(-d).l2g(lwi);
                        if(ls.ok)
                        {
                            sh.ok = true;
                            sh.o = ls.o;
                            sh.d = ls.d;
                            sh.t1 = ls.t1;
                            sh.beta = ls.li;
                            sh.medium = ls.t1 > 1 ? S.vacuum_medium : medium_id;
                            sh.seed = shadow_stream_seed(stage_a, stage_b, 1);
                        }
                        if(!zero3(phase))
                        {
                            alive = true;
                            n_o = spos;
                            n_d = nrm(nd);
                            n_beta_le = beta * phase;
                            n_beta = n_beta_le / pv;
                            n_pdf = pv;
                            n_medium = medium_id;
                        }
                        else
                            splat(film, S.width, px, py, rad);
                    }
                }
            }
        }

        // ---------------- shade stage (shade.cpp:29-235)
        const uint64_t shade_a = smp.word_a(), shade_b = smp.word_b();
        if(!h.hit)
        {
            V3f le(0.0f);
            if(S.env_type)
            {
                const V3f L = env_le(P, d);
                if(bsdf_pdf < 0)
                    le = beta_le * L / -bsdf_pdf;
                else
                    le = beta_le * L / (bsdf_pdf + (1.0f / NL) * env_pdf(P, d));
            }
            splat(film, S.width, px, py, scattered ? le : le + rad);
        }
        else
        {
            const int inst = static_cast<int>(h.inst);
            const float *l2w = S.inst_l2w + inst * 12, *w2l = S.inst_w2l + inst * 12;
            const int geo = S.inst_geo[inst];
            const uint64_t ti = S.geo_offset[geo] + h.prim;
            auto shd = [&](int k) {
                const float *q = S.shade + (static_cast<uint64_t>(k) * S.total_geo_tris + ti) * 4;
                return V3f(q[0], q[1], q[2]);
            };
            // get_hitinfo (core/btrc/core/scene.cpp:9-64)
            const V3f pos = o + h.t * d;
            Frame<float> gf(shd(0), shd(1), shd(2));
            gf.x = nrm(vec(l2w, gf.x));
            gf.y = nrm(vec(l2w, gf.y));
            gf.z = nrm(nor(w2l, gf.z));
            const V3f interp = nrm(nor(w2l, shd(3) + shd(4) * h.b1 + shd(5) * h.b2));
            // texture coordinate (core/btrc/core/scene.cpp:48-51)
            auto shw = [&](int k) { return S.shade[(static_cast<uint64_t>(k) * S.total_geo_tris + ti) * 4 + 3]; };
            const float tu = shw(0) + shw(1) * h.b1 + shw(2) * h.b2;
            const float tv = shw(3) + shw(4) * h.b1 + shw(5) * h.b2;

            V3f le(0.0f);
            const int light = S.inst_light[inst];
            if(light >= 0)
            {
                const V3f I(S.light_intensity[light * 3], S.light_intensity[light * 3 + 1], S.light_intensity[light * 3 + 2]);
                const V3f e = dot(gf.z, -d) >= 0 ? I : V3f(0.0f);
                if(bsdf_pdf < 0)
                    le = beta_le * e / -bsdf_pdf;
                else
                {
                    float pdf_li = 0;
                    const V3f to_ref = o - pos;
                    if(dot(gf.z, to_ref) > 0)
                    {
                        const float sc = S.light_scale[light];
                        const float d2 = dot(to_ref, to_ref);
                        const float d3 = std::sqrt(d2) * d2;
                        pdf_li = 1.0f / (sc * sc) * (1.0f / S.geo_area_total[S.light_geo[light]]) * d3 /
                                 std::fabs(dot(gf.z, to_ref));
                    }
                    le = beta_le * e / (bsdf_pdf + (1.0f / NL) * pdf_li);
                }
            }
            if(scattered)
                splat(film, S.width, px, py, le);
            else
            {
                rad = rad + le;
                if(russian_roulette(S, beta, depth, smp))
                    splat(film, S.width, px, py, rad);
                else
                {
                    LightSample ls = sample_light(P, pos, gf.z, true, smp);
                    float mr[20];
                    std::memcpy(mr, S.mat + S.inst_mat[inst] * 20, sizeof(mr));
                    const int mtype = static_cast<int>(mr[0]);
                    const bool term = mr[1] != 0.0f;
                    ShadeFrame fr;
                    fr.g = gf;
                    fr.s = gf.rotate_to_new_z(interp);
                    // textured parameters and the normal map (material/utils/normal_map.cpp:13-21)
                    const int trow = S.mat_texrow ? S.mat_texrow[S.inst_mat[inst]] : -1;
                    if(trow >= 0)
                    {
                        const OMatTex &mt = static_cast<const OMatTex *>(S.mat_tex)[trow];
                        if(mt.prog[0] >= 0)
                        {
                            const V3f c = otex_eval(S, mt.prog[0], tu, tv);
                            mr[2] = c.x;
                            mr[3] = c.y;
                            mr[4] = c.z;
                        }
                        for(int k = 3; k < 16; ++k)
                            if(mt.prog[k] >= 0)
                                mr[2 + k] = otex_eval(S, mt.prog[k], tu, tv).x;
                        if(mt.normal >= 0)
                        {
                            const V3f ln = 2.0f * otex_eval(S, mt.normal, tu, tv) - V3f(1.0f);
                            fr.s = fr.s.rotate_to_new_z(nrm(fr.s.l2g(ln)));
                        }
                    }
                    Mat<float> M;
                    if(mtype <= 2)
                        M.init(mtype, mr + 2);
                    // g-buffer at the first hit (shade.cpp:133-139, 195-202): black has
                    // albedo 0, invisible 1, the others their colour; black and invisible
                    // report the geometric normal, the others the shading normal
                    if(depth == 0 && aov)
                    {
                        const V3f alb = mtype == 3 ? V3f(0.0f) : mtype == 4 ? V3f(1.0f) : V3f(mr[2], mr[3], mr[4]);
                        const V3f nv = (mtype == 3 || mtype == 4) ? gf.z : fr.s.z;
                        if(std::isfinite(alb.x) && std::isfinite(alb.y) && std::isfinite(alb.z) &&
                           std::isfinite(nv.x) && std::isfinite(nv.y) && std::isfinite(nv.z))
                        {
                            double *q = aov + (static_cast<size_t>(py) * S.width + px) * 6;
                            q[0] += alb.x; q[1] += alb.y; q[2] += alb.z;
                            q[3] += nv.x; q[4] += nv.y; q[5] += nv.z;
                        }
                    }
                    float u0, u1, u2;
                    smp.get3d(u0, u1, u2);
                    const V3f wo = -d;
                    CS<float> bs;
                    auto eval = [&](V3f wi) -> V3f {
                        if(mtype > 2)
                            return V3f(0.0f);
                        const ShadeFrame f = fr.flip(wo);
                        const V3f lwi = nrm(f.s.g2l(wi)), lwo = nrm(f.s.g2l(wo));
                        float k = f.corr(wi);
                        if(term)
                            k *= fr.term(wi);
                        return M.eval(lwi, lwo) * k;
                    };
                    auto pdf = [&](V3f wi) -> float {
                        if(mtype > 2)
                            return 0.0f;
                        const ShadeFrame f = fr.flip(wo);
                        return M.pdf(nrm(f.s.g2l(wi)), nrm(f.s.g2l(wo)));
                    };
                    if(mtype == 4)
                    {
                        // invisible.cpp: pass straight through
                        bs.f = V3f(1.0f / std::fabs(dot(gf.z, nrm(wo))));
                        bs.dir = -wo;
                        bs.pdf = 1;
                        bs.delta = true;
                    }
                    else if(mtype == 6)
                    {
                        // glass.cpp:34-95
                        const ShadeFrame f = fr.flip(wo);
                        const V3f col(mr[2], mr[3], mr[4]);
                        const float ior = mr[5];
                        const V3f nwo = nrm(f.s.g2l(wo));
                        const float F = diel_fresnel(ior, 1.0f, nwo.z);
                        if(u0 < F)
                        {
                            const V3f lwi(-nwo.x, -nwo.y, nwo.z);
                            const V3f wi = f.s.l2g(lwi);
                            if(!fr.black(wi))
                            {
                                bs.f = col * F / std::fabs(lwi.z) * f.corr(wi);
                                bs.dir = wi;
                                bs.pdf = F;
                                bs.delta = true;
                            }
                        }
                        else
                        {
                            const float nz = nwo.z > 0 ? 1.0f : -1.0f;
                            const float eta = nwo.z > 0 ? 1.0f / ior : ior;
                            const float cti = std::fabs(nwo.z);
                            const float s2i = std::max(0.0f, 1.0f - cti * cti);
                            const float s2t = eta * eta * s2i;
                            if(s2t < 1)
                            {
                                const float ctt = std::sqrt(1.0f - s2t);
                                const V3f nwi = nrm((eta * cti - ctt) * V3f(0, 0, nz) - eta * nwo);
                                const V3f wi = f.s.l2g(nwi);
                                if(!fr.black(wi))
                                {
                                    bs.f = col * (eta * eta * (1.0f - F) / std::fabs(nwi.z)) * f.corr(wi);
                                    bs.dir = wi;
                                    bs.pdf = 1.0f - diel_fresnel(ior, 1.0f, nwi.z);
                                    bs.delta = true;
                                }
                            }
                        }
                    }
                    else if(mtype == 5)
                    {
                        // mirror.cpp
                        const ShadeFrame f = fr.flip(wo);
                        V3f lwo = f.s.g2l(wo);
                        if(lwo.z > 0)
                        {
                            lwo = nrm(lwo);
                            const V3f wi = f.s.l2g(V3f(-lwo.x, -lwo.y, lwo.z));
                            if(!fr.black(wi))
                            {
                                const V3f col(mr[2], mr[3], mr[4]);
                                bs.f = schlick3(col, lwo.z) / lwo.z * f.corr(wi);
                                bs.dir = wi;
                                bs.pdf = 1;
                                bs.delta = true;
                            }
                        }
                    }
                    else if(mtype <= 2)
                    {
                        // BSDFAggregate::sample (aggregate.cpp:32-105)
                        const ShadeFrame f = fr.flip(wo);
                        const V3f lwo = nrm(f.s.g2l(wo));
                        const CS<float> c = M.sample(lwo, u0, u1, u2);
                        if(c.pdf > 0)
                        {
                            const V3f wi = f.s.l2g(c.dir);
                            if(!fr.black(wi))
                            {
                                float k = f.corr(wi);
                                if(term)
                                    k *= fr.term(wi);
                                bs.f = c.f * k;
                                bs.dir = wi;
                                bs.pdf = c.pdf;
                            }
                        }
                    }
                    V3f sf(0.0f);
                    float spdf = 0;
                    if(ls.ok)
                    {
                        sf = eval(ls.d);
                        ls.ok = !zero3(sf);
                        if(ls.ok)
                            spdf = pdf(ls.d);
                    }
                    if(ls.ok)
                    {
                        const bool sout = dot(gf.z, ls.d) > 0, lout = dot(gf.z, d) < 0;
                        sh.ok = true;
                        sh.o = ls.o;
                        sh.d = ls.d;
                        sh.t1 = ls.t1;
                        sh.medium = sout == lout ? ray_medium : (sout ? S.inst_outer[inst] : S.inst_inner[inst]);
                        const float c = std::fabs(dot(nrm(ls.d), gf.z));
                        sh.beta = ls.li * beta * sf * c / (spdf + ls.pdf);
                        sh.seed = shadow_stream_seed(shade_a, shade_b, 2);
                    }
                    if(zero3(bs.f))
                        splat(film, S.width, px, py, rad);
                    else
                    {
                        const V3f nd = nrm(bs.dir);
                        const float c = std::fabs(dot(nd, gf.z));
                        alive = true;
                        n_beta_le = beta * c * bs.f;
                        n_beta = n_beta_le / bs.pdf;
                        n_o = ioffset_dir(pos, gf.z, nd);
                        n_d = nd;
                        n_medium = dot(gf.z, nd) > 0 ? S.inst_outer[inst] : S.inst_inner[inst];
                        n_pdf = bs.delta ? -bs.pdf : bs.pdf;
                    }
                }
            }
        }

        // ---------------- shadow stage (shadow.cpp:24-76)
        if(sh.ok)
        {
            const float so[3] = { sh.o.x, sh.o.y, sh.o.z }, sdir[3] = { sh.d.x, sh.d.y, sh.d.z };
            if(!P.bvh.any(so, sdir, sh.t1))
            {
                V3f b = sh.beta;
                if(P.has_media)
                {
                    PcgSmp shadow_rng;
                    shadow_rng.p.seed(sh.seed, PCG_STREAM);
                    if(sh.t1 > 1)
                        b = b * medium_tr(S, medium(S, S.vacuum_medium), sh.o, sh.o + nrm(sh.d) * S.world_diagonal,
                                          shadow_rng);
                    else
                        b = b * medium_tr(S, medium(S, sh.medium), sh.o, sh.o + sh.d * sh.t1, shadow_rng);
                }
                splat(film, S.width, px, py, b);
            }
        }
        if(!alive)
            return;
        o = n_o;
        d = n_d;
        t1 = FMAX;
        beta = n_beta;
        beta_le = n_beta_le;
        bsdf_pdf = n_pdf;
        ray_medium = n_medium;
        ++depth;
    }
}

} // namespace

// ------------------------------------------------------------------ wide-BVH work counts
// The closest-hit traversal of the library's exported 8-wide BVH (80-byte nodes,
// 48-byte triangle records; layout in btrc_gb300/csrc/layout.h), restated sequentially:
// node groups visited in the kernel's child order (slot XOR ray octant), child boxes
// dequantised and slab-tested exactly in FP64 against the current closest t, every
// triangle of a hit leaf tested with the watertight test. The counts are the traversal's
// algorithmic work on these rays: node visits and triangle tests with exact box tests and
// no deferred triangle rounds (the kernel pads its FP32 box tests and tests triangles in
// pooled rounds, so it can only do more).
namespace {

struct WideCount
{
    uint32_t nodes = 0, tris = 0;
};

WideCount wide_count(const uint8_t *nodes, const float *tris, const float *o, const float *d, float t1)
{
    WideCount c;
    const WRay wr = make_wray(o, d);
    const int octant = (d[0] < 0) | ((d[1] < 0) << 1) | ((d[2] < 0) << 2);
    const uint32_t oct_inv = static_cast<uint32_t>(7 - octant);
    double inv[3];
    for(int a = 0; a < 3; ++a)
    {
        const double dd = std::fabs(d[a]) < 1e-20 ? std::copysign(1e-20, static_cast<double>(d[a])) : d[a];
        inv[a] = 1.0 / dd;
    }
    float best = t1;
    uint32_t stack_x[64], stack_y[64];
    int sp = 0;
    uint32_t ngx = 0, ngy = 0x80000000u;
    for(;;)
    {
        uint32_t tgx = 0, tgy = 0;
        if(ngy > 0x00ffffffu)
        {
            int bit = 31;
            while(!((ngy >> bit) & 1u))
                --bit;
            const uint32_t slot = (static_cast<uint32_t>(bit) - 24u) ^ oct_inv;
            const uint32_t below = slot ? (ngy & ((1u << slot) - 1u) & 0xffu) : 0u;
            const uint32_t ni = ngx + static_cast<uint32_t>(__builtin_popcount(below));
            ngy &= ~(1u << bit);
            if(ngy > 0x00ffffffu && sp < 64)
            {
                stack_x[sp] = ngx;
                stack_y[sp] = ngy;
                ++sp;
            }
            ++c.nodes;
            const uint8_t *nd = nodes + static_cast<size_t>(ni) * 80;
            float px[3];
            std::memcpy(px, nd, 12);
            uint32_t child_base, tri_base;
            std::memcpy(&child_base, nd + 16, 4);
            std::memcpy(&tri_base, nd + 20, 4);
            const uint8_t imask = nd[15];
            uint32_t hm = 0;
            for(int sl = 0; sl < 8; ++sl)
            {
                const uint32_t m = nd[24 + sl];
                if(!m)
                    continue;
                double tmin = 0.0, tmax = best;
                for(int a = 0; a < 3; ++a)
                {
                    const double scale = std::ldexp(1.0, static_cast<int>(nd[12 + a]) - 127);
                    const double lo = px[a] + nd[32 + a * 8 + sl] * scale, hi = px[a] + nd[56 + a * 8 + sl] * scale;
                    const double ta = (lo - o[a]) * inv[a], tb = (hi - o[a]) * inv[a];
                    tmin = std::max(tmin, std::min(ta, tb));
                    tmax = std::min(tmax, std::max(ta, tb));
                }
                if(tmin <= tmax)
                {
                    const bool inner = (m & 0x18u) == 0x18u;
                    const uint32_t b = inner ? ((m & 0x1fu) ^ oct_inv) : (m & 0x1fu);
                    hm |= (m >> 5) << b;
                }
            }
            ngx = child_base;
            ngy = (hm & 0xff000000u) | imask;
            tgx = tri_base;
            tgy = hm & 0x00ffffffu;
        }
        while(tgy)
        {
            int tb = 31;
            while(!((tgy >> tb) & 1u))
                --tb;
            tgy &= ~(1u << tb);
            const float *r = tris + static_cast<size_t>(tgx + static_cast<uint32_t>(tb)) * 12;
            ++c.tris;
            float t, b1, b2;
            if(watertight(wr, r, r + 4, r + 8, best, t, b1, b2))
                best = std::min(best, t);
        }
        if(ngy <= 0x00ffffffu)
        {
            if(!sp)
                break;
            --sp;
            ngx = stack_x[sp];
            ngy = stack_y[sp];
        }
    }
    return c;
}

} // namespace

extern "C" {

// transmittance of segments (a, b: 6 floats each) through one medium of the scene, each
// with its own PCG stream seeded (seeds[i], PCG_STREAM): the independent-sampler stream
// the library's medium test hook uses
void oracle_medium_tr_batch(const OracleScene *S, int medium_id, const float *seg, const uint64_t *seeds, uint64_t n,
                            float *out)
{
    const Med m = medium(*S, medium_id);
    for(uint64_t i = 0; i < n; ++i)
    {
        PcgSmp smp;
        smp.p.seed(seeds[i], PCG_STREAM);
        const V3f a(seg[i * 6 + 0], seg[i * 6 + 1], seg[i * 6 + 2]);
        const V3f b(seg[i * 6 + 3], seg[i * 6 + 4], seg[i * 6 + 5]);
        out[i] = medium_tr(*S, m, a, b, smp).x;
    }
}

// node visits and triangle tests of the exported wide BVH per ray (see wide_count)
void oracle_wide_bvh_counts(const uint8_t *nodes, const float *tris, const float *rays, uint64_t n,
                            uint32_t *node_visits, uint32_t *tri_tests, int threads)
{
    parallel_for(n, threads, [&](uint64_t i) {
        const float *r = rays + i * 8;
        const WideCount c = wide_count(nodes, tris, r, r + 4, r[7]);
        node_visits[i] = c.nodes;
        tri_tests[i] = c.tris;
    });
}

void *oracle_bvh_build(const float *tris, const uint32_t *ids, uint64_t n)
{
    auto *b = new Bvh();
    b->build(tris, ids, n);
    return b;
}

void oracle_bvh_free(void *b) { delete static_cast<Bvh *>(b); }

// rays: 8 floats each (o.xyz, medium, d.xyz, t1); hits: 4 floats (t, prim bits, b1, b2)
void oracle_trace_closest(const void *bvh, const float *rays, uint64_t m, uint32_t *flags, float *hits, int threads)
{
    const Bvh &B = *static_cast<const Bvh *>(bvh);
    parallel_for(m, threads, [&](uint64_t i) {
        const float *r = rays + i * 8;
        const Bvh::Hit h = B.closest(r, r + 4, r[7]);
        flags[i] = h.hit ? (h.inst | (1u << 30)) : 0u;
        float *o = hits + i * 4;
        o[0] = h.hit ? h.t : 0.0f;
        const uint32_t prim = h.hit ? h.prim : 0u;
        std::memcpy(&o[1], &prim, 4);
        o[2] = h.hit ? h.b1 : 0.0f;
        o[3] = h.hit ? h.b2 : 0.0f;
    });
}

void oracle_trace_any(const void *bvh, const float *rays, uint64_t m, uint32_t *occ, int threads)
{
    const Bvh &B = *static_cast<const Bvh *>(bvh);
    parallel_for(m, threads, [&](uint64_t i) {
        const float *r = rays + i * 8;
        occ[i] = B.any(r, r + 4, r[7]) ? 1u : 0u;
    });
}

void oracle_sampler_batch(int type, int width, int height, const uint32_t *pixel_xy, const uint32_t *sample_index,
                          uint64_t n, uint32_t dims, float *out)
{
    const Sampler::HC hc = Sampler::consts(width, height);
    for(uint64_t i = 0; i < n; ++i)
    {
        Sampler s;
        s.init(type, hc, pixel_xy[i] & 0xffffu, pixel_xy[i] >> 16, sample_index[i]);
        for(uint32_t k = 0; k < dims; ++k)
            out[i * dims + k] = s.get1d();
    }
}

// PCG32 raw output stream for the published known-answer test
void oracle_pcg32_stream(uint64_t initstate, uint64_t initseq, uint32_t n, uint32_t *out)
{
    Pcg p;
    p.seed(initstate, initseq);
    for(uint32_t i = 0; i < n; ++i)
        out[i] = p.next();
}

uint64_t oracle_murmur64a(const uint8_t *key, uint64_t len, uint64_t seed) { return murmur64a(key, len, seed); }

// FP64 local-space BSDF: material records of 16 floats (p[0..14], type in [15])
// op 0: out 4 doubles (f.rgb, pdf); op 1: out 7 doubles (f.rgb, pdf, wi.xyz)
void oracle_bsdf_batch(int op, const float *mat, const double *wo, const double *wu, uint64_t n, double *out)
{
    for(uint64_t i = 0; i < n; ++i)
    {
        Mat<double> M;
        M.init(static_cast<int>(mat[i * 16 + 15]), mat + i * 16);
        const V<double> lwo(wo[i * 3], wo[i * 3 + 1], wo[i * 3 + 2]);
        if(op == 0)
        {
            const V<double> lwi(wu[i * 3], wu[i * 3 + 1], wu[i * 3 + 2]);
            const V<double> f = M.eval(lwi, lwo);
            out[i * 4 + 0] = f.x;
            out[i * 4 + 1] = f.y;
            out[i * 4 + 2] = f.z;
            out[i * 4 + 3] = M.pdf(lwi, lwo);
        }
        else if(op == 2)
        {
            // the sampled direction alone, before Disney's bad-sample rejection
            M.keep_bad = true;
            const CS<double> s = M.sample(lwo, wu[i * 3], wu[i * 3 + 1], wu[i * 3 + 2]);
            const bool ok = !(s.dir.x == 0 && s.dir.y == 0 && s.dir.z == 0);
            out[i * 7 + 0] = ok ? 1.0 : 0.0;
            out[i * 7 + 1] = out[i * 7 + 2] = out[i * 7 + 3] = 0.0;
            out[i * 7 + 4] = s.dir.x;
            out[i * 7 + 5] = s.dir.y;
            out[i * 7 + 6] = s.dir.z;
        }
        else
        {
            const CS<double> s = M.sample(lwo, wu[i * 3], wu[i * 3 + 1], wu[i * 3 + 2]);
            out[i * 7 + 0] = s.f.x;
            out[i * 7 + 1] = s.f.y;
            out[i * 7 + 2] = s.f.z;
            out[i * 7 + 3] = s.pdf;
            out[i * 7 + 4] = s.dir.x;
            out[i * 7 + 5] = s.dir.y;
            out[i * 7 + 6] = s.dir.z;
        }
    }
}

// The same restatement instantiated in FP32 (inputs rounded to float first): the
// spread between this and the FP64 result is the conditioning of the formula itself.
void oracle_bsdf_batch_f32(int op, const float *mat, const double *wo, const double *wu, uint64_t n, double *out)
{
    for(uint64_t i = 0; i < n; ++i)
    {
        Mat<float> M;
        M.init(static_cast<int>(mat[i * 16 + 15]), mat + i * 16);
        const V<float> lwo(float(wo[i * 3]), float(wo[i * 3 + 1]), float(wo[i * 3 + 2]));
        if(op == 0)
        {
            const V<float> lwi(float(wu[i * 3]), float(wu[i * 3 + 1]), float(wu[i * 3 + 2]));
            const V<float> f = M.eval(lwi, lwo);
            out[i * 4 + 0] = f.x;
            out[i * 4 + 1] = f.y;
            out[i * 4 + 2] = f.z;
            out[i * 4 + 3] = M.pdf(lwi, lwo);
        }
        else
        {
            const CS<float> s = M.sample(lwo, float(wu[i * 3]), float(wu[i * 3 + 1]), float(wu[i * 3 + 2]));
            out[i * 7 + 0] = s.f.x;
            out[i * 7 + 1] = s.f.y;
            out[i * 7 + 2] = s.f.z;
            out[i * 7 + 3] = s.pdf;
            out[i * 7 + 4] = s.dir.x;
            out[i * 7 + 5] = s.dir.y;
            out[i * 7 + 6] = s.dir.z;
        }
    }
}

void *oracle_prepare(const OracleScene *S)
{
    auto *P = new Prepared();
    P->S = S;
    P->bvh.build(S->tris, S->ids, S->ntri);
    P->geo_alias.resize(S->ngeo);
    for(int l = 0; l < S->nlight; ++l)
    {
        const int g = S->light_geo[l];
        if(!P->geo_alias[g].accept.empty())
            continue;
        std::vector<float> a(S->tri_area + S->geo_offset[g], S->tri_area + S->geo_offset[g] + S->geo_count[g]);
        P->geo_alias[g].init(a);
    }
    if(S->filter == 1)
    {
        // GaussianFilter::commit (film_filter/gaussian.cpp:27-52)
        const float r = S->filter_radius, al = S->filter_alpha;
        const float expv = std::exp(-al * r * r);
        auto gau = [&](float x) { return std::max(0.0f, std::exp(-al * x * x) - expv); };
        std::vector<float> v(256 * 256, 0.0f);
        for(int y = 0; y < 256; ++y)
        {
            const float yf = 2 * r * (y + 0.5f) / 256 - r;
            for(int x = 0; x < 256; ++x)
            {
                const float xf = 2 * r * (x + 0.5f) / 256 - r;
                if(xf * xf + yf * yf < r * r)
                    v[y * 256 + x] = gau(xf) * gau(yf);
            }
        }
        P->filter.init(v);
    }
    P->hc = Sampler::consts(S->width, S->height);
    if(S->env_type == 2)
    {
        P->env_frame = Frame<float>::from_z(V3f(S->env_up[0], S->env_up[1], S->env_up[2]));
        build_env_table(*P);
    }
    P->has_media = S->nvol > 0;
    for(int i = 0; i < S->ninst && S->nmed > 0; ++i)
        if(medium(*S, S->inst_inner[i]).type != 0 || medium(*S, S->inst_outer[i]).type != 0)
            P->has_media = true;
    return P;
}

void oracle_release(void *p) { delete static_cast<Prepared *>(p); }

// Render the pixel range [pixel_begin, pixel_end) with samples [sample_begin, sample_end)
// into film (4 doubles per pixel of the full image: rgb sum, weight). Threads split pixels.
void oracle_render(const void *prepared, uint64_t pixel_begin, uint64_t pixel_end, uint32_t sample_begin,
                   uint32_t sample_end, double *film, int threads)
{
    const Prepared &P = *static_cast<const Prepared *>(prepared);
    const uint64_t pixels = static_cast<uint64_t>(P.S->width) * P.S->height;
    parallel_for(pixel_end - pixel_begin, threads, [&](uint64_t k) {
        const uint64_t pix = pixel_begin + k;
        for(uint32_t s = sample_begin; s < sample_end; ++s)
            trace_path(P, static_cast<uint64_t>(s) * pixels + pix, film);
    });
}

// the same with the first-hit g-buffer: aov holds 6 doubles per pixel (albedo sum,
// normal sum); weights are in film[3]
void oracle_render_aov(const void *prepared, uint64_t pixel_begin, uint64_t pixel_end, uint32_t sample_begin,
                       uint32_t sample_end, double *film, double *aov, int threads)
{
    const Prepared &P = *static_cast<const Prepared *>(prepared);
    const uint64_t pixels = static_cast<uint64_t>(P.S->width) * P.S->height;
    parallel_for(pixel_end - pixel_begin, threads, [&](uint64_t k) {
        const uint64_t pix = pixel_begin + k;
        for(uint32_t s = sample_begin; s < sample_end; ++s)
            trace_path(P, static_cast<uint64_t>(s) * pixels + pix, film, aov);
    });
}

} // extern "C"
