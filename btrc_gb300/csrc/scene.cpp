#include "scene.h"
#include "taskpool.h"

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <map>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <thread>

namespace bt {

// ---------------------------------------------------------------- Mat4 / Transform

Mat4 Mat4::identity() { return rows(1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1); }

Mat4 Mat4::rows(float m00, float m01, float m02, float m03,
                float m10, float m11, float m12, float m13,
                float m20, float m21, float m22, float m23,
                float m30, float m31, float m32, float m33)
{
    Mat4 r;
    r.a[0][0] = m00; r.a[0][1] = m01; r.a[0][2] = m02; r.a[0][3] = m03;
    r.a[1][0] = m10; r.a[1][1] = m11; r.a[1][2] = m12; r.a[1][3] = m13;
    r.a[2][0] = m20; r.a[2][1] = m21; r.a[2][2] = m22; r.a[2][3] = m23;
    r.a[3][0] = m30; r.a[3][1] = m31; r.a[3][2] = m32; r.a[3][3] = m33;
    return r;
}

Mat4 Mat4::translate(float x, float y, float z)
{
    return rows(1, 0, 0, x, 0, 1, 0, y, 0, 0, 1, z, 0, 0, 0, 1);
}

Mat4 Mat4::scale(float x, float y, float z)
{
    return rows(x, 0, 0, 0, 0, y, 0, 0, 0, 0, z, 0, 0, 0, 0, 1);
}

// The reference fills its column-major storage with the textbook Rodrigues entries
// (common/btrc/utils/math/mat4.cpp:117-145), so at(r, c) holds entry [c][r] of the
// textbook matrix. That is reproduced here: R below is the textbook matrix, stored
// transposed.
Mat4 Mat4::rotate(V3 axis, float rad)
{
    const V3 a = normalize(axis);
    const float s = std::sin(rad), c = std::cos(rad);
    float R[3][3];
    R[0][0] = a.x * a.x + (1 - a.x * a.x) * c;
    R[0][1] = a.x * a.y * (1 - c) - a.z * s;
    R[0][2] = a.x * a.z * (1 - c) + a.y * s;
    R[1][0] = a.x * a.y * (1 - c) + a.z * s;
    R[1][1] = a.y * a.y + (1 - a.y * a.y) * c;
    R[1][2] = a.y * a.z * (1 - c) - a.x * s;
    R[2][0] = a.x * a.z * (1 - c) - a.y * s;
    R[2][1] = a.y * a.z * (1 - c) + a.x * s;
    R[2][2] = a.z * a.z + (1 - a.z * a.z) * c;
    return rows(R[0][0], R[1][0], R[2][0], 0,
                R[0][1], R[1][1], R[2][1], 0,
                R[0][2], R[1][2], R[2][2], 0,
                0, 0, 0, 1);
}

Mat4 Mat4::rotate_x(float rad)
{
    const float S = std::sin(rad), C = std::cos(rad);
    return rows(1, 0, 0, 0, 0, C, -S, 0, 0, S, C, 0, 0, 0, 0, 1);
}

Mat4 Mat4::rotate_y(float rad)
{
    const float S = std::sin(rad), C = std::cos(rad);
    return rows(C, 0, S, 0, 0, 1, 0, 0, -S, 0, C, 0, 0, 0, 0, 1);
}

Mat4 Mat4::rotate_z(float rad)
{
    const float S = std::sin(rad), C = std::cos(rad);
    return rows(C, -S, 0, 0, S, C, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1);
}

Mat4 operator*(const Mat4 &a, const Mat4 &b)
{
    Mat4 r;
    for(int i = 0; i < 4; ++i)
        for(int j = 0; j < 4; ++j)
            r.a[i][j] = a.a[i][0] * b.a[0][j] + a.a[i][1] * b.a[1][j] +
                        a.a[i][2] * b.a[2][j] + a.a[i][3] * b.a[3][j];
    return r;
}

Transform operator*(const Transform &a, const Transform &b)
{
    Transform r;
    r.mat = a.mat * b.mat;
    r.inv = b.inv * a.inv;
    return r;
}

V3 Transform::point(V3 p) const
{
    return V3(mat.a[0][0] * p.x + mat.a[0][1] * p.y + mat.a[0][2] * p.z + mat.a[0][3],
              mat.a[1][0] * p.x + mat.a[1][1] * p.y + mat.a[1][2] * p.z + mat.a[1][3],
              mat.a[2][0] * p.x + mat.a[2][1] * p.y + mat.a[2][2] * p.z + mat.a[2][3]);
}

V3 Transform::vector(V3 v) const
{
    return V3(mat.a[0][0] * v.x + mat.a[0][1] * v.y + mat.a[0][2] * v.z,
              mat.a[1][0] * v.x + mat.a[1][1] * v.y + mat.a[1][2] * v.z,
              mat.a[2][0] * v.x + mat.a[2][1] * v.y + mat.a[2][2] * v.z);
}

V3 Transform::normal(V3 n) const
{
    return V3(inv.a[0][0] * n.x + inv.a[1][0] * n.y + inv.a[2][0] * n.z,
              inv.a[0][1] * n.x + inv.a[1][1] * n.y + inv.a[2][1] * n.z,
              inv.a[0][2] * n.x + inv.a[1][2] * n.y + inv.a[2][2] * n.z);
}

void Transform::to_affine(float l2w[12], float w2l[12]) const
{
    for(int r = 0; r < 3; ++r)
        for(int c = 0; c < 4; ++c)
        {
            l2w[r * 4 + c] = mat.a[r][c];
            w2l[r * 4 + c] = inv.a[r][c];
        }
}

// factory/btrc/factory/node/node.cpp:166-214. An array composes later elements on the
// left: ret = elem * ret. rotate_z keeps the reference's (mat, inv) pair as written
// (common/btrc/utils/math/transform.cpp:111-114: both use rotate_z(-rad)).
Transform parse_transform(const json::NodeP &n)
{
    Transform t;
    if(n->is_array())
    {
        for(auto &e : n->elems)
            t = parse_transform(e) * t;
        return t;
    }
    if(auto c = n->find("translate"))
    {
        const V3 v = json::as_vec3(c);
        t.mat = Mat4::translate(v.x, v.y, v.z);
        t.inv = Mat4::translate(-v.x, -v.y, -v.z);
        return t;
    }
    if(auto c = n->find("rotate"))
    {
        const V3 axis = json::as_vec3(c->child("axis"));
        const float rad = json::as_radian(c->child("angle"));
        t.mat = Mat4::rotate(axis, rad);
        t.inv = Mat4::rotate(axis, -rad);
        return t;
    }
    if(auto c = n->find("rotate_x"))
    {
        const float rad = json::as_radian(c);
        t.mat = Mat4::rotate_x(rad);
        t.inv = Mat4::rotate_x(-rad);
        return t;
    }
    if(auto c = n->find("rotate_y"))
    {
        const float rad = json::as_radian(c);
        t.mat = Mat4::rotate_y(rad);
        t.inv = Mat4::rotate_y(-rad);
        return t;
    }
    if(auto c = n->find("rotate_z"))
    {
        const float rad = json::as_radian(c);
        t.mat = Mat4::rotate_z(-rad);
        t.inv = Mat4::rotate_z(-rad);
        return t;
    }
    if(auto c = n->find("scale"))
    {
        const V3 s = json::as_vec3(c);
        t.mat = Mat4::scale(s.x, s.y, s.z);
        t.inv = Mat4::scale(1 / s.x, 1 / s.y, 1 / s.z);
        return t;
    }
    throw json::ParseError("unknown transform3d type");
}

// ---------------------------------------------------------------- alias tables

std::vector<AliasEntry8> build_alias_table(const std::vector<float> &probs)
{
    if(probs.empty())
        throw std::runtime_error("alias table over an empty distribution");
    double dsum = 0;
    for(float p : probs)
        dsum += p;
    const float sum = static_cast<float>(dsum);
    if(!(sum > 0))
        throw std::runtime_error("alias table over a zero distribution");
    const float ratio = static_cast<float>(probs.size()) / sum;
    std::vector<AliasEntry8> units(probs.size());
    std::vector<uint32_t> overs, unders;
    for(uint32_t i = 0; i < units.size(); ++i)
    {
        const float p = probs[i] * ratio;
        units[i].accept = p;
        units[i].alias = i;
        if(p > 1)
            overs.push_back(i);
        else if(p < 1)
            unders.push_back(i);
    }
    while(!overs.empty() && !unders.empty())
    {
        const uint32_t over = overs.back();
        const uint32_t under = unders.back();
        overs.pop_back();
        unders.pop_back();
        units[over].accept -= 1 - units[under].accept;
        units[under].alias = over;
        if(units[over].accept > 1)
            overs.push_back(over);
        else if(units[over].accept < 1)
            unders.push_back(over);
    }
    for(auto i : overs)
        units[i].accept = 1;
    for(auto i : unders)
        units[i].accept = 1;
    return units;
}

std::vector<AliasEntry8> build_gaussian_filter_table(float radius, float alpha)
{
    const float expv = std::exp(-alpha * radius * radius);
    auto gaussian = [&](float d) { return std::max(0.0f, std::exp(-alpha * d * d) - expv); };
    std::vector<float> values(FILTER_GRID * FILTER_GRID, 0.0f);
    for(int y = 0; y < FILTER_GRID; ++y)
    {
        const float yf = 2 * radius * (y + 0.5f) / FILTER_GRID - radius;
        for(int x = 0; x < FILTER_GRID; ++x)
        {
            const float xf = 2 * radius * (x + 0.5f) / FILTER_GRID - radius;
            if(xf * xf + yf * yf < radius * radius)
                values[y * FILTER_GRID + x] = gaussian(xf) * gaussian(yf);
        }
    }
    return build_alias_table(values);
}

// ---------------------------------------------------------------- camera

Camera make_pinhole(V3 eye, V3 dst, V3 up, float fov_y_deg, float w_over_h)
{
    const V3 forward = normalize(dst - eye);
    const V3 ex = normalize(cross(forward, up));
    const V3 ey = normalize(cross(forward, ex));
    const float y_len = 2 * std::tan(0.5f * fov_y_deg * PI / 180);
    const float x_len = w_over_h * y_len;
    Camera c;
    c.eye = eye;
    c.lbc = eye + forward - 0.5f * (x_len * ex + y_len * ey);
    c.film_x = x_len * ex;
    c.film_y = y_len * ey;
    return c;
}

// ---------------------------------------------------------------- OBJ loading

namespace {

struct ObjIndex { int v, vt, vn; };

inline const char *skip_spaces(const char *p)
{
    while(*p == ' ' || *p == '\t')
        ++p;
    return p;
}

bool parse_obj_index(const char *&p, ObjIndex &out)
{
    out = { 0, 0, 0 };
    char *end;
    long v = std::strtol(p, &end, 10);
    if(end == p)
        return false;
    out.v = static_cast<int>(v);
    p = end;
    if(*p == '/')
    {
        ++p;
        if(*p != '/')
        {
            long t = std::strtol(p, &end, 10);
            if(end != p)
            {
                out.vt = static_cast<int>(t);
                p = end;
            }
        }
        if(*p == '/')
        {
            ++p;
            long n = std::strtol(p, &end, 10);
            if(end != p)
            {
                out.vn = static_cast<int>(n);
                p = end;
            }
        }
    }
    return true;
}

inline int resolve_obj(int idx, size_t count)
{
    // 1-based positive, or negative relative to the end; 0 means absent
    if(idx > 0)
        return idx - 1;
    if(idx < 0)
        return static_cast<int>(count) + idx;
    return -1;
}

// common/btrc/utils/math/triangle.h: triangle_dpdu
V3 triangle_dpdu(V3 B_A, V3 C_A, float bax, float bay, float cax, float cay, V3 nor)
{
    const float m00 = bax, m01 = bay, m10 = cax, m11 = cay;
    const float det = m00 * m11 - m01 * m10;
    if(det == 0.0f)
        return Frame::from_z(nor).x;
    const float inv_det = 1 / det;
    return normalize(m11 * inv_det * B_A - m01 * inv_det * C_A);
}

} // namespace

HostGeometry geometry_from_arrays(const std::string &name, std::vector<V3> positions, const std::vector<V3> &normals,
                                  const std::vector<float> &uvs, const std::vector<ObjIndex> &corners,
                                  bool to_unit_cube);

namespace {

// One line-aligned piece of an OBJ file: what it holds (first pass) and where its
// records go in the whole file's arrays (second pass).
struct ObjChunk
{
    const char *begin, *end;
    size_t nv = 0, nvn = 0, nvt = 0, ncorner = 0;    // counts in this chunk
    size_t v0 = 0, vn0 = 0, vt0 = 0, corner0 = 0;    // records before this chunk
    std::string error;
};

inline bool is_v(const char *l) { return l[0] == 'v' && (l[1] == ' ' || l[1] == '\t'); }
inline bool is_f(const char *l) { return l[0] == 'f' && (l[1] == ' ' || l[1] == '\t'); }

// vertices of a face line (without parsing the numbers)
size_t face_vertex_count(const char *q, const char *eol)
{
    size_t n = 0;
    for(;;)
    {
        q = skip_spaces(q);
        if(q >= eol || *q == '\r' || *q == '\n')
            return n;
        ++n;
        while(q < eol && *q != ' ' && *q != '\t' && *q != '\r' && *q != '\n')
            ++q;
    }
}

void obj_count(ObjChunk &c)
{
    for(const char *p = c.begin; p < c.end;)
    {
        const char *line = skip_spaces(p);
        const char *eol = static_cast<const char *>(std::memchr(line, '\n', c.end - line));
        if(!eol)
            eol = c.end;
        if(is_v(line))
            ++c.nv;
        else if(line[0] == 'v' && line[1] == 'n')
            ++c.nvn;
        else if(line[0] == 'v' && line[1] == 't')
            ++c.nvt;
        else if(is_f(line))
        {
            const size_t k = face_vertex_count(line + 2, eol);
            if(k >= 3)
                c.ncorner += 3 * (k - 2);
        }
        p = eol + 1;
    }
}

void obj_parse(ObjChunk &c, V3 *positions, V3 *normals, float *uvs, ObjIndex *corners)
{
    size_t nv = c.v0, nvn = c.vn0, nvt = c.vt0, nc = c.corner0;
    ObjIndex face[64];
    std::vector<ObjIndex> big;
    for(const char *p = c.begin; p < c.end;)
    {
        const char *line = skip_spaces(p);
        const char *eol = static_cast<const char *>(std::memchr(line, '\n', c.end - line));
        if(!eol)
            eol = c.end;
        if(is_v(line))
        {
            char *e;
            const float x = std::strtof(line + 2, &e);
            const float y = std::strtof(e, &e);
            const float z = std::strtof(e, &e);
            positions[nv++] = V3(x, y, z);
        }
        else if(line[0] == 'v' && line[1] == 'n')
        {
            char *e;
            const float x = std::strtof(line + 3, &e);
            const float y = std::strtof(e, &e);
            const float z = std::strtof(e, &e);
            normals[nvn++] = V3(x, y, z);
        }
        else if(line[0] == 'v' && line[1] == 't')
        {
            char *e;
            const float u = std::strtof(line + 3, &e);
            const float v = std::strtof(e, &e);
            uvs[2 * nvt] = u;
            uvs[2 * nvt + 1] = v;
            ++nvt;
        }
        else if(is_f(line))
        {
            const size_t k = face_vertex_count(line + 2, eol);
            ObjIndex *f = face;
            if(k > 64)
            {
                big.resize(k);
                f = big.data();
            }
            const char *q = line + 2;
            for(size_t j = 0; j < k; ++j)
            {
                q = skip_spaces(q);
                if(!parse_obj_index(q, f[j]))
                {
                    c.error = "bad face";
                    return;
                }
                // negative indices count back from the records read so far
                f[j].v = resolve_obj(f[j].v, nv);
                f[j].vt = resolve_obj(f[j].vt, nvt);
                f[j].vn = resolve_obj(f[j].vn, nvn);
            }
            if(k < 3)
            {
                c.error = "invalid obj face vertex count";
                return;
            }
            for(size_t j = 1; j + 1 < k; ++j)
            {
                corners[nc++] = f[0];
                corners[nc++] = f[j];
                corners[nc++] = f[j + 1];
            }
        }
        p = eol + 1;
    }
}

} // namespace

// OBJ meshes are parsed in two passes over line-aligned pieces of the file, in
// parallel: the first counts the records of each piece, the second parses every piece
// into its place (negative indices resolve against the records before the face, as in
// a sequential read), so the result does not depend on the number of threads.
HostGeometry load_obj(const std::string &filename, bool to_unit_cube)
{
    std::ifstream fin(filename, std::ios::binary | std::ios::ate);
    if(!fin)
        throw std::runtime_error("cannot open obj file '" + filename + "'");
    std::string text(static_cast<size_t>(fin.tellg()), '\0');
    fin.seekg(0);
    fin.read(&text[0], static_cast<std::streamsize>(text.size()));

    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t pieces = std::max<size_t>(1, std::min<size_t>(hw * 4, text.size() / (1u << 18)));
    std::vector<ObjChunk> chunks;
    const char *base = text.data(), *tend = base + text.size();
    const char *p = base;
    for(size_t k = 0; k < pieces && p < tend; ++k)
    {
        const char *e = k + 1 == pieces ? tend : std::min(tend, base + text.size() * (k + 1) / pieces);
        if(e < tend)
        {
            const char *nl = static_cast<const char *>(std::memchr(e, '\n', tend - e));
            e = nl ? nl + 1 : tend;
        }
        if(e > p)
            chunks.push_back(ObjChunk{ p, e });
        p = e;
    }
    // the pool of a batch load when there is one, else threads of our own
    std::unique_ptr<TaskPool> own;
    TaskPool *pp = current_pool();
    if(!pp)
    {
        own = std::make_unique<TaskPool>(static_cast<int>(std::min<size_t>(hw, chunks.size())));
        pp = own.get();
    }
    TaskPool &pool = *pp;
    pool.parallel_for(chunks.size(), 1, [&](size_t b, size_t e) {
        for(size_t k = b; k < e; ++k)
            obj_count(chunks[k]);
    });
    size_t nv = 0, nvn = 0, nvt = 0, nc = 0;
    for(auto &c : chunks)
    {
        c.v0 = nv;
        c.vn0 = nvn;
        c.vt0 = nvt;
        c.corner0 = nc;
        nv += c.nv;
        nvn += c.nvn;
        nvt += c.nvt;
        nc += c.ncorner;
    }
    std::vector<V3> positions(nv), normals(nvn);
    std::vector<float> uvs(2 * nvt);
    std::vector<ObjIndex> corners(nc);  // 3 per triangle, already resolved to 0-based (-1 absent)
    pool.parallel_for(chunks.size(), 1, [&](size_t b, size_t e) {
        for(size_t k = b; k < e; ++k)
            obj_parse(chunks[k], positions.data(), normals.data(), uvs.data(), corners.data());
    });
    for(auto &c : chunks)
        if(!c.error.empty())
            throw std::runtime_error(c.error + " in obj file '" + filename + "'");

    for(auto &c : corners)
    {
        if(c.v < 0 || static_cast<size_t>(c.v) >= positions.size())
            throw std::runtime_error("invalid obj vertex index: out of range");
        if(c.vn >= 0 && static_cast<size_t>(c.vn) >= normals.size())
            throw std::runtime_error("invalid obj normal index: out of range");
        if(c.vt >= 0 && static_cast<size_t>(c.vt) * 2 + 1 >= uvs.size())
            throw std::runtime_error("invalid obj tex coord index: out of range");
    }

    return geometry_from_arrays(filename, std::move(positions), normals, uvs, corners, to_unit_cube);
}

HostGeometry geometry_from_arrays(const std::string &name, std::vector<V3> positions, const std::vector<V3> &normals,
                                  const std::vector<float> &uvs, const std::vector<ObjIndex> &corners,
                                  bool to_unit_cube)
{
    const std::string &filename = name;
    if(to_unit_cube && !positions.empty())
    {
        // common/btrc/utils/triangle_mesh_loader.cpp:195-213
        V3 lo(MAX_FLOAT), hi(-MAX_FLOAT);
        for(auto &q : positions)
        {
            lo = vmin(lo, q);
            hi = vmax(hi, q);
        }
        const V3 ext = hi - lo;
        const float emax = std::max(ext.x, std::max(ext.y, ext.z));
        const float s = emax > 0 ? 1 / emax : 1.0f;
        for(auto &q : positions)
            q = s * (q - 0.5f * (lo + hi));
    }

    HostGeometry g;
    g.filename = filename;
    const size_t ntri = corners.size() / 3;
    g.pos.resize(ntri * 3);
    for(auto &s : g.shade)
        s.resize(ntri);
    g.area.resize(ntri);
    g.bmin = V3(MAX_FLOAT);
    g.bmax = V3(-MAX_FLOAT);
    for(auto &q : positions)
    {
        g.bmin = vmin(g.bmin, q);
        g.bmax = vmax(g.bmax, q);
    }
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    std::unique_ptr<TaskPool> own;
    TaskPool *pp = current_pool();
    if(!pp)
    {
        own = std::make_unique<TaskPool>(ntri >= (1u << 16) ? static_cast<int>(hw) : 1);
        pp = own.get();
    }
    TaskPool &pool = *pp;
    pool.parallel_for(ntri, 1u << 13, [&](size_t tb, size_t te) {
    for(size_t i = tb; i < te; ++i)
    {
        const ObjIndex *c = &corners[i * 3];
        const V3 a = positions[c[0].v], b = positions[c[1].v], cc = positions[c[2].v];
        g.pos[i * 3 + 0] = a;
        g.pos[i * 3 + 1] = b;
        g.pos[i * 3 + 2] = cc;
        const V3 geo_z = normalize(cross(b - a, cc - a));
        V3 sz[3];
        float tu[3], tv[3];
        for(int k = 0; k < 3; ++k)
        {
            if(c[k].vn < 0)
                sz[k] = geo_z;
            else
            {
                sz[k] = normals[c[k].vn];
                if(sz[k].x == 0.0f && sz[k].y == 0.0f && sz[k].z == 0.0f)
                    sz[k] = geo_z;
            }
            if(c[k].vt < 0)
            {
                tu[k] = 0;
                tv[k] = 0;
            }
            else
            {
                tu[k] = uvs[c[k].vt * 2];
                tv[k] = uvs[c[k].vt * 2 + 1];
            }
        }
        const V3 gx = triangle_dpdu(b - a, cc - a, tu[1] - tu[0], tv[1] - tv[0],
                                    tu[2] - tu[0], tv[2] - tv[0], geo_z);
        const V3 gz = geo_z;
        const V3 gy = normalize(cross(gz, gx));
        g.shade[0][i] = { gx.x, gx.y, gx.z, tu[0] };
        g.shade[1][i] = { gy.x, gy.y, gy.z, tu[1] - tu[0] };
        g.shade[2][i] = { gz.x, gz.y, gz.z, tu[2] - tu[0] };
        g.shade[3][i] = { sz[0].x, sz[0].y, sz[0].z, tv[0] };
        const V3 sba = sz[1] - sz[0], sca = sz[2] - sz[0];
        g.shade[4][i] = { sba.x, sba.y, sba.z, tv[1] - tv[0] };
        g.shade[5][i] = { sca.x, sca.y, sca.z, tv[2] - tv[0] };
        g.area[i] = 0.5f * length(cross(b - a, cc - a));
    }
    });
    double total = 0;
    for(size_t i = 0; i < ntri; ++i)
        total += g.area[i];
    g.total_area = static_cast<float>(total);
    return g;
}

// ---------------------------------------------------------------- procedural geometry

// Inline geometry creators (an extension; the reference reads triangle meshes from OBJ
// files only): "sphere" (icosphere of radius 1, `subdivisions` 0..8, smooth normals,
// spherical texture coordinates), "quad" (unit square in the xz plane facing +y, texture
// coordinates over [0,1]^2) and "box" (the cube [-0.5, 0.5]^3 facing outwards, flat).
// Built in double precision and rounded once.
HostGeometry procedural_geometry(const std::string &type, int subdivisions)
{
    std::vector<V3> pos, nor;
    std::vector<float> uvs;
    std::vector<ObjIndex> corners;
    if(type == "sphere")
    {
        if(subdivisions < 0 || subdivisions > 8)
            throw std::runtime_error("sphere subdivisions must be within 0..8");
        const double t = (1.0 + std::sqrt(5.0)) / 2.0;
        std::vector<std::array<double, 3>> v = { { -1, t, 0 }, { 1, t, 0 }, { -1, -t, 0 }, { 1, -t, 0 },
                                                 { 0, -1, t }, { 0, 1, t }, { 0, -1, -t }, { 0, 1, -t },
                                                 { t, 0, -1 }, { t, 0, 1 }, { -t, 0, -1 }, { -t, 0, 1 } };
        auto unit = [](std::array<double, 3> p) {
            const double l = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
            return std::array<double, 3>{ p[0] / l, p[1] / l, p[2] / l };
        };
        for(auto &p : v)
            p = unit(p);
        std::vector<std::array<int, 3>> f = { { 0, 11, 5 }, { 0, 5, 1 },  { 0, 1, 7 },   { 0, 7, 10 }, { 0, 10, 11 },
                                              { 1, 5, 9 },  { 5, 11, 4 }, { 11, 10, 2 }, { 10, 7, 6 }, { 7, 1, 8 },
                                              { 3, 9, 4 },  { 3, 4, 2 },  { 3, 2, 6 },   { 3, 6, 8 },  { 3, 8, 9 },
                                              { 4, 9, 5 },  { 2, 4, 11 }, { 6, 2, 10 },  { 8, 6, 7 },  { 9, 8, 1 } };
        for(int level = 0; level < subdivisions; ++level)
        {
            std::map<std::pair<int, int>, int> cache;
            auto mid = [&](int a, int b) {
                const auto key = a < b ? std::make_pair(a, b) : std::make_pair(b, a);
                auto it = cache.find(key);
                if(it != cache.end())
                    return it->second;
                v.push_back(unit({ v[a][0] + v[b][0], v[a][1] + v[b][1], v[a][2] + v[b][2] }));
                const int id = static_cast<int>(v.size()) - 1;
                cache[key] = id;
                return id;
            };
            std::vector<std::array<int, 3>> nf;
            nf.reserve(f.size() * 4);
            for(auto &tri : f)
            {
                const int a = tri[0], b = tri[1], c = tri[2];
                const int ab = mid(a, b), bc = mid(b, c), ca = mid(c, a);
                nf.push_back({ a, ab, ca });
                nf.push_back({ b, bc, ab });
                nf.push_back({ c, ca, bc });
                nf.push_back({ ab, bc, ca });
            }
            f.swap(nf);
        }
        const double PI_D = 3.14159265358979323846;
        for(auto &p : v)
        {
            pos.emplace_back(static_cast<float>(p[0]), static_cast<float>(p[1]), static_cast<float>(p[2]));
            nor.push_back(pos.back());
            uvs.push_back(static_cast<float>(std::atan2(p[2], p[0]) / (2 * PI_D) + 0.5));
            uvs.push_back(static_cast<float>(std::acos(std::max(-1.0, std::min(1.0, p[1]))) / PI_D));
        }
        for(auto &tri : f)
            for(int k = 0; k < 3; ++k)
                corners.push_back({ tri[k], tri[k], tri[k] });
    }
    else if(type == "quad")
    {
        pos = { V3(-0.5f, 0, -0.5f), V3(0.5f, 0, -0.5f), V3(0.5f, 0, 0.5f), V3(-0.5f, 0, 0.5f) };
        uvs = { 0, 0, 1, 0, 1, 1, 0, 1 };
        for(int k : { 0, 2, 1, 0, 3, 2 })
            corners.push_back({ k, k, -1 });
    }
    else if(type == "box")
    {
        for(int c = 0; c < 8; ++c)
            pos.emplace_back((c & 4) ? 0.5f : -0.5f, (c & 2) ? 0.5f : -0.5f, (c & 1) ? 0.5f : -0.5f);
        // two outward-facing triangles per face (vertex index = 4 x + 2 y + z)
        const int faces[12][3] = { { 0, 1, 3 }, { 0, 3, 2 }, { 4, 6, 7 }, { 4, 7, 5 }, { 0, 4, 5 }, { 0, 5, 1 },
                                   { 2, 3, 7 }, { 2, 7, 6 }, { 0, 2, 6 }, { 0, 6, 4 }, { 1, 5, 7 }, { 1, 7, 3 } };
        for(auto &tri : faces)
            for(int k = 0; k < 3; ++k)
                corners.push_back({ tri[k], -1, -1 });
    }
    else
        throw std::runtime_error("unsupported geometry type '" + type + "'");
    return geometry_from_arrays("<" + type + ">", std::move(pos), nor, uvs, corners, false);
}

// ---------------------------------------------------------------- scene file

namespace {

using json::NodeP;

std::string resolve_path(const std::string &p, const std::string &scene_dir)
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

// Material parameters from Texture2D nodes: constants go to p[k]; other textures compile
// to programs recorded in the material's MaterialTex row (k = 0 is the RGB colour).
struct ParamSink
{
    TexStore &T;
    Material &m;
    MaterialTex &mt;
    bool textured = false;

    void spectrum(int k, const NodeP &n)
    {
        V3 c;
        const int prog = compile_texture2d(T, n, c);
        if(prog < 0)
        {
            m.p[k] = c.x; m.p[k + 1] = c.y; m.p[k + 2] = c.z;
        }
        else
        {
            mt.prog[k] = prog;
            textured = true;
        }
    }
    // a float parameter reads the texture's red channel (Texture2D::sample_float)
    void scalar(int k, const NodeP &n, float def_if_null)
    {
        if(!n)
        {
            m.p[k] = def_if_null;
            return;
        }
        V3 c;
        const int prog = compile_texture2d(T, n, c);
        if(prog < 0)
            m.p[k] = c.x;
        else
        {
            mt.prog[k] = prog;
            textured = true;
        }
    }
};

Material make_material(const NodeP &n, TexStore &T, std::vector<MaterialTex> &rows)
{
    Material m{};
    MaterialTex mt;
    for(int &k : mt.prog)
        k = -1;
    mt.normal = -1;
    mt.pad[0] = mt.pad[1] = mt.pad[2] = 0;
    ParamSink P{ T, m, mt };
    const std::string type = json::as_string(n->child("type"));
    m.shadow_terminator = json::bool_or(n, "shadow_terminator_term", true) ? 1 : 0;
    // NormalMap::load (builtin/btrc/builtin/material/utils/normal_map.cpp:5-11): the
    // "normal" texture of diffuse, metal, disney, glass and mirror
    if(type == "diffuse" || type == "metal" || type == "disney" || type == "glass" || type == "mirror")
    {
        if(auto nn = n->find("normal"))
        {
            V3 c;
            const int prog = compile_texture2d(T, nn, c);
            if(prog < 0)
            {
                // a constant normal map: one instruction holding the constant
                TexInstr ins{};
                ins.op = TEXOP_CONST;
                ins.a[0] = c.x; ins.a[1] = c.y; ins.a[2] = c.z;
                TexInstr end{};
                end.op = TEXOP_END;
                mt.normal = static_cast<int>(T.instr.size());
                T.instr.push_back(ins);
                T.instr.push_back(end);
            }
            else
                mt.normal = prog;
            P.textured = true;
        }
    }
    if(type == "diffuse")
    {
        m.type = MAT_DIFFUSE;
        P.spectrum(0, n->child("color"));
    }
    else if(type == "metal")
    {
        // builtin/btrc/builtin/material/metal.cpp:50-78
        m.type = MAT_METAL;
        P.spectrum(0, n->child("color"));
        P.scalar(3, n->child("roughness"), 0);
        P.scalar(4, n->find("anisotropic"), 0);
    }
    else if(type == "disney")
    {
        // builtin/btrc/builtin/material/disney.cpp:844-894 creator defaults
        m.type = MAT_DISNEY;
        P.spectrum(0, n->child("color"));
        P.scalar(3, n->child("metallic"), 0);
        P.scalar(4, n->child("roughness"), 0);
        P.scalar(5, n->find("specular"), 1);
        P.scalar(6, n->find("specular_tint"), 0);
        P.scalar(7, n->find("anisotropic"), 0);
        P.scalar(8, n->find("sheen"), 0);
        P.scalar(9, n->find("sheen_tint"), 0);
        P.scalar(10, n->find("clearcoat"), 0);
        P.scalar(11, n->find("clearcoat_gloss"), 1);
        P.scalar(12, n->find("transmission"), 0);
        // transmission_roughness defaults to the roughness texture
        P.scalar(13, n->find("transmission_roughness") ? n->find("transmission_roughness") : n->child("roughness"), 0);
        P.scalar(14, n->find("ior"), 1.5f);
    }
    else if(type == "black")
        m.type = MAT_BLACK;
    else if(type == "invisible")
        m.type = MAT_INVISIBLE;
    else if(type == "mirror")
    {
        m.type = MAT_MIRROR;
        P.spectrum(0, n->child("color"));
    }
    else if(type == "glass")
    {
        // builtin/btrc/builtin/material/glass.cpp:117-129
        m.type = MAT_GLASS;
        P.spectrum(0, n->child("color"));
        P.scalar(3, n->child("ior"), 1.5f);
    }
    else
        throw std::runtime_error("unsupported material type '" + type + "'");
    m.tex = -1;
    if(P.textured)
    {
        m.tex = static_cast<int32_t>(rows.size());
        rows.push_back(mt);
    }
    return m;
}

struct GridData
{
    int w = 1, h = 1, d = 1;
    int ch = 1;               // channels kept in v: 1, or 3 (rgb of a 3- or 4-channel array)
    std::vector<float> v;     // x fastest, channels interleaved
    V3 rgb = V3(0);           // the value of a constant texture
    float constant = 0;       // rgb.x
    bool is_constant = true;
};

// Texture3D: constant value / spectrum, {"type":"constant","value":...} or
// {"type":"array","text":file} (common/btrc/utils/cuda/array.cpp:313-384), plus
// {"type":"array","binary":file}: raw header "BTG1" int32 w h d then float32 x-fastest.
// Text arrays keep channel 0 unless keep_rgb; "byte" components are read as one
// character each and mapped as signed 8-bit normalised values, as the reference's
// `uint8_t comp; fin >> comp` + SNorm8 texture format do.
GridData load_texture3d(const NodeP &n, const std::string &scene_dir, bool keep_rgb = false)
{
    GridData g;
    if(n->is_value() || n->is_array())
    {
        g.rgb = json::as_spectrum(n);
        g.constant = g.rgb.x;
        return g;
    }
    const std::string type = json::as_string(n->child("type"));
    if(type == "constant")
    {
        g.rgb = json::as_spectrum(n->child("value"));
        g.constant = g.rgb.x;
        return g;
    }
    if(type != "array")
        throw std::runtime_error("unsupported texture3d type '" + type + "'");
    g.is_constant = false;
    if(auto b = n->find("binary"))
    {
        const std::string fn = resolve_path(json::as_string(b), scene_dir);
        std::ifstream f(fn, std::ios::binary);
        if(!f)
            throw std::runtime_error("failed to open file: " + fn);
        char magic[4];
        int32_t dims[3];
        f.read(magic, 4);
        f.read(reinterpret_cast<char *>(dims), sizeof(dims));
        if(!f || std::memcmp(magic, "BTG1", 4) != 0 || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0)
            throw std::runtime_error("bad binary grid header: " + fn);
        g.w = dims[0]; g.h = dims[1]; g.d = dims[2];
        g.v.resize(static_cast<size_t>(g.w) * g.h * g.d);
        f.read(reinterpret_cast<char *>(g.v.data()), g.v.size() * sizeof(float));
        if(!f)
            throw std::runtime_error("truncated binary grid: " + fn);
        return g;
    }
    const std::string fn = resolve_path(json::as_string(n->child("text")), scene_dir);
    std::ifstream f(fn);
    if(!f)
        throw std::runtime_error("failed to open file: " + fn);
    std::string comp;
    int ch;
    f >> comp >> ch >> g.w >> g.h >> g.d;
    if(!f || g.w <= 0 || g.h <= 0 || g.d <= 0)
        throw std::runtime_error("Array::load_from_text: failed to parse file head");
    if(ch != 1 && ch != 3 && ch != 4)
        throw std::runtime_error("unsupported channel count: " + std::to_string(ch));
    if(comp != "float" && comp != "byte")
        throw std::runtime_error("unknown component type: " + comp);
    g.ch = keep_rgb && ch > 1 ? 3 : 1;
    const size_t texels = static_cast<size_t>(g.w) * g.h * g.d;
    g.v.resize(texels * g.ch);
    for(size_t i = 0; i < texels; ++i)
    {
        for(int c = 0; c < ch; ++c)
        {
            float val;
            if(comp == "float")
                f >> val;
            else
            {
                char cc;
                f >> cc;
                const int u = static_cast<int>(static_cast<unsigned char>(cc));
                const int sv = u >= 128 ? u - 256 : u;
                val = std::max(static_cast<float>(sv) / 127.0f, -1.0f);
            }
            if(c < g.ch)
                g.v[i * g.ch + c] = val;
        }
    }
    if(!f)
        throw std::runtime_error("failed to load " + fn);
    return g;
}

// VolumePrimitive::get_bounding_box (core/btrc/core/volume.cpp:54-68): the box of o and
// o + x, o + y, o + z, as the reference computes it
V3 volume_box_lower(const VolumePrim &v)
{
    const V3 o(v.o[0], v.o[1], v.o[2]), x(v.x[0], v.x[1], v.x[2]), y(v.y[0], v.y[1], v.y[2]),
        z(v.z[0], v.z[1], v.z[2]);
    return vmin(vmin(o, o + x), vmin(o + y, o + z));
}

V3 volume_box_upper(const VolumePrim &v)
{
    const V3 o(v.o[0], v.o[1], v.o[2]), x(v.x[0], v.x[1], v.x[2]), y(v.y[0], v.y[1], v.y[2]),
        z(v.z[0], v.z[1], v.z[2]);
    return vmax(vmax(o, o + x), vmax(o + y, o + z));
}

// all eight corners: the box the volume BVH is built over. The reference builds its BVH
// over the four-point box above, which for a sheared volume leaves parts of it outside its
// node bounds; bounding all corners makes the overlap set exactly the volumes containing
// the point (the two boxes agree for axis-aligned volumes)
void volume_corner_box(const VolumePrim &v, V3 &lo, V3 &hi)
{
    const V3 o(v.o[0], v.o[1], v.o[2]), x(v.x[0], v.x[1], v.x[2]), y(v.y[0], v.y[1], v.y[2]),
        z(v.z[0], v.z[1], v.z[2]);
    lo = V3(MAX_FLOAT);
    hi = V3(-MAX_FLOAT);
    for(int c = 0; c < 8; ++c)
    {
        const V3 p = o + ((c & 1) ? x : V3(0)) + ((c & 2) ? y : V3(0)) + ((c & 4) ? z : V3(0));
        lo = vmin(lo, p);
        hi = vmax(hi, p);
    }
}

VolumePrim make_volume(const NodeP &n, int id, const std::string &scene_dir, std::vector<float> &pool)
{
    VolumePrim v{};
    v.id = id;
    const V3 o = json::as_vec3(n->child("o")), x = json::as_vec3(n->child("x")), y = json::as_vec3(n->child("y")),
             z = json::as_vec3(n->child("z"));
    const V3 *axes[3] = { &x, &y, &z };
    float *dst[3] = { v.x, v.y, v.z };
    float *dstd[3] = { v.xd, v.yd, v.zd };
    float *inv[3] = { &v.x_inv_len2, &v.y_inv_len2, &v.z_inv_len2 };
    v.o[0] = o.x; v.o[1] = o.y; v.o[2] = o.z;
    for(int a = 0; a < 3; ++a)
    {
        const V3 e = *axes[a];
        const float l2 = length_square(e);
        if(!(l2 > 0))
            throw std::runtime_error("degenerate volume axis");
        dst[a][0] = e.x; dst[a][1] = e.y; dst[a][2] = e.z;
        *inv[a] = 1.0f / l2;
        const V3 ed = e / l2;
        dstd[a][0] = ed.x; dstd[a][1] = ed.y; dstd[a][2] = ed.z;
    }
    GridData sig = load_texture3d(n->child("sigma_t"), scene_dir);
    if(sig.is_constant)
    {
        v.sigma_offset = -1;
        v.sigma_const = sig.constant;
        v.sigma_max = sig.constant;
        v.sres[0] = v.sres[1] = v.sres[2] = 1;
    }
    else
    {
        v.sigma_offset = static_cast<int32_t>(pool.size());
        v.sres[0] = sig.w; v.sres[1] = sig.h; v.sres[2] = sig.d;
        float mx = -MAX_FLOAT;
        for(float s : sig.v)
            mx = std::max(mx, s);
        v.sigma_max = mx;
        pool.insert(pool.end(), sig.v.begin(), sig.v.end());
    }
    GridData alb = load_texture3d(n->child("albedo"), scene_dir, true);
    if(alb.is_constant)
    {
        v.albedo_offset = -1;
        v.albedo_const[0] = alb.rgb.x; v.albedo_const[1] = alb.rgb.y; v.albedo_const[2] = alb.rgb.z;
        v.ares[0] = v.ares[1] = v.ares[2] = 1;
        v.albedo_channels = 3;
    }
    else
    {
        v.albedo_offset = static_cast<int32_t>(pool.size());
        v.ares[0] = alb.w; v.ares[1] = alb.h; v.ares[2] = alb.d;
        v.albedo_channels = alb.ch;
        pool.insert(pool.end(), alb.v.begin(), alb.v.end());
    }
    if(pool.size() > static_cast<size_t>(INT32_MAX))
        throw std::runtime_error("volume grids exceed 2^31 floats");
    return v;
}

// Binary BVH over the volume boxes: object-median splits on the widest centroid axis,
// leaves of at most 4 boxes, children of a node stored next to each other. The depth
// stays below log2(n) + 1, far inside the traversal stack (VOL_STACK).
void build_volume_bvh(const std::vector<VolumePrim> &in, std::vector<VolumePrim> &out, std::vector<VolNode> &nodes)
{
    out.clear();
    nodes.clear();
    if(in.empty())
        return;
    std::vector<V3> lo(in.size()), hi(in.size()), c(in.size());
    for(size_t i = 0; i < in.size(); ++i)
    {
        volume_corner_box(in[i], lo[i], hi[i]);
        c[i] = 0.5f * (lo[i] + hi[i]);
    }
    std::vector<int> idx(in.size());
    std::iota(idx.begin(), idx.end(), 0);
    nodes.emplace_back();
    struct Task { int node, b, e; };
    std::vector<Task> todo{ { 0, 0, static_cast<int>(in.size()) } };
    while(!todo.empty())
    {
        const Task t = todo.back();
        todo.pop_back();
        V3 bl(MAX_FLOAT), bh(-MAX_FLOAT), cl(MAX_FLOAT), ch(-MAX_FLOAT);
        for(int i = t.b; i < t.e; ++i)
        {
            bl = vmin(bl, lo[idx[i]]);
            bh = vmax(bh, hi[idx[i]]);
            cl = vmin(cl, c[idx[i]]);
            ch = vmax(ch, c[idx[i]]);
        }
        VolNode &nd = nodes[t.node];
        nd.lower[0] = bl.x; nd.lower[1] = bl.y; nd.lower[2] = bl.z;
        nd.upper[0] = bh.x; nd.upper[1] = bh.y; nd.upper[2] = bh.z;
        if(t.e - t.b <= 4)
        {
            nd.prim_beg = static_cast<int32_t>(out.size());
            for(int i = t.b; i < t.e; ++i)
                out.push_back(in[idx[i]]);
            nd.prim_end = static_cast<int32_t>(out.size());
            continue;
        }
        const V3 ext = ch - cl;
        const int axis = ext.x >= ext.y && ext.x >= ext.z ? 0 : (ext.y >= ext.z ? 1 : 2);
        const int mid = (t.b + t.e) / 2;
        std::nth_element(idx.begin() + t.b, idx.begin() + mid, idx.begin() + t.e, [&](int a, int b) {
            const float ca = axis == 0 ? c[a].x : (axis == 1 ? c[a].y : c[a].z);
            const float cb = axis == 0 ? c[b].x : (axis == 1 ? c[b].y : c[b].z);
            return ca < cb || (ca == cb && a < b);
        });
        const int left = static_cast<int>(nodes.size());
        nd.prim_beg = -1;
        nd.prim_end = left;
        nodes.emplace_back();
        nodes.emplace_back();
        todo.push_back({ left + 1, mid, t.e });
        todo.push_back({ left, t.b, mid });
    }
}

struct MediumBuilder
{
    std::string scene_dir;
    std::vector<HostMedium> media;
    std::map<const json::Node *, int> pool;

    int create(const NodeP &n)
    {
        auto it = pool.find(n.get());
        if(it != pool.end())
            return it->second;
        HostMedium m{};
        build(n, Transform{}, false, m);
        media.push_back(std::move(m));
        const int id = static_cast<int>(media.size()) - 1;
        pool[n.get()] = id;
        return id;
    }

    void build(const NodeP &n, const Transform &w2l, bool has_xf, HostMedium &m)
    {
        const std::string type = json::as_string(n->child("type"));
        if(type == "transform")
        {
            Transform t;
            if(auto tn = n->find("world_to_local"))
                t = parse_transform(tn);
            else
            {
                Transform l2w = parse_transform(n->child("local_to_world"));
                t.mat = l2w.inv;
                t.inv = l2w.mat;
            }
            // nested transforms compose: the outer one is applied first
            build(n->child("medium"), has_xf ? t * w2l : t, true, m);
            return;
        }
        float l2w_a[12], w2l_a[12];
        w2l.to_affine(w2l_a, l2w_a);
        std::memcpy(m.dev.w2l, w2l_a, sizeof(w2l_a));
        std::memcpy(m.dev.l2w, l2w_a, sizeof(l2w_a));
        m.priority = json::float_or(n, "priority", 0.0f);
        m.dev.priority = static_cast<int32_t>(m.priority);
        if(type == "homogeneous")
        {
            m.dev.type = MED_HOMOGENEOUS;
            m.dev.sigma_t_const = json::as_float(n->child("sigma_t"));
            const V3 a = json::as_spectrum(n->child("albedo"));
            m.dev.albedo[0] = a.x; m.dev.albedo[1] = a.y; m.dev.albedo[2] = a.z;
            m.dev.g = json::float_or(n, "g", 0.0f);
        }
        else if(type == "hetergeneous" || type == "heterogeneous")
        {
            m.dev.type = MED_HETEROGENEOUS;
            GridData sig = load_texture3d(n->child("sigma_t"), scene_dir);
            GridData alb = load_texture3d(n->child("albedo"), scene_dir, true);
            if(!alb.is_constant)
                throw std::runtime_error("only constant medium albedo is supported");
            const V3 a = alb.rgb;
            m.dev.albedo[0] = a.x; m.dev.albedo[1] = a.y; m.dev.albedo[2] = a.z;
            if(auto gn = n->find("g"))
            {
                GridData gg = load_texture3d(gn, scene_dir);
                if(!gg.is_constant)
                    throw std::runtime_error("only constant phase g is supported");
                m.dev.g = gg.constant;
            }
            if(sig.is_constant)
            {
                m.grid.assign(1, sig.constant);
                m.dev.res_x = m.dev.res_y = m.dev.res_z = 1;
            }
            else
            {
                m.grid = std::move(sig.v);
                m.dev.res_x = sig.w; m.dev.res_y = sig.h; m.dev.res_z = sig.d;
            }
            float mx = 0;
            for(float v : m.grid)
                mx = std::max(mx, v);
            m.dev.sigma_max = std::max(mx, 0.001f);
        }
        else
            throw std::runtime_error("unsupported medium type '" + type + "'");
    }
};

} // namespace

HostScene load_scene(const std::string &path)
{
    HostScene S;
    S.path = path;
    const std::string scene_dir = std::filesystem::absolute(std::filesystem::path(path)).parent_path().string();
    NodeP root = json::parse_scene_file(path, scene_dir);

    S.params.width = json::as_int(root->child("width"));
    S.params.height = json::as_int(root->child("height"));
    if(S.params.width <= 0 || S.params.height <= 0 || S.params.width > 65535 || S.params.height > 65535)
        throw std::runtime_error("film size out of range");

    // camera (builtin/btrc/builtin/camera/pinhole.cpp:101-114)
    {
        NodeP cam = root->child("camera");
        const std::string type = json::as_string(cam->child("type"));
        if(type != "pinhole")
            throw std::runtime_error("unsupported camera type '" + type + "'");
        S.camera = make_pinhole(json::as_vec3(cam->child("eye")), json::as_vec3(cam->child("dst")),
                                json::as_vec3(cam->child("up")), json::as_degree(cam->child("fov_y")),
                                static_cast<float>(S.params.width) / S.params.height);
    }

    // post_processors: one group or an array of them
    if(auto pp = root->find("post_processors"))
    {
        std::vector<NodeP> items;
        if(pp->is_group())
            items.push_back(pp);
        else if(pp->is_array())
            items = pp->elems;
        else
            throw std::runtime_error("parse_post_processors: array or group is expected");
        for(const NodeP &n : items)
        {
            PostProcess q;
            const std::string type = json::as_string(n->child("type"));
            auto path_or_empty = [&](const char *key) {
                auto c = n->find(key);
                if(!c)
                    return std::string();
                const std::string v = json::as_string(c);
                return v.empty() ? v : resolve_path(v, scene_dir);
            };
            if(type == "save")
            {
                q.type = POST_SAVE;
                q.gamma = json::float_or(n, "gamma", 1.0f);
                q.color = path_or_empty("color");
                q.albedo = path_or_empty("albedo");
                q.normal = path_or_empty("normal");
            }
            else if(type == "tonemap")
            {
                q.type = POST_TONEMAP;
                q.exposure = json::float_or(n, "exposure", 1.0f);
            }
            else if(type == "denoise")
                q.type = POST_DENOISE;
            else
                throw std::runtime_error("unsupported post processor type '" + type + "'");
            S.post.push_back(q);
        }
    }

    // renderer (builtin/btrc/builtin/renderer/wavefront.cpp:375-397)
    {
        NodeP r = root->child("renderer");
        RenderParams &P = S.params;
        P.renderer_type = json::as_string(r->child("type"));
        if(P.renderer_type != "wfpt" && P.renderer_type != "pt")
            throw std::runtime_error("unsupported renderer type '" + P.renderer_type + "'");
        P.tile = json::bool_or(r, "tile", P.tile);
        P.spp = json::int_or(r, "spp", P.spp);
        P.min_depth = json::int_or(r, "min_depth", P.min_depth);
        P.max_depth = json::int_or(r, "max_depth", P.max_depth);
        P.rr_threshold = json::float_or(r, "rr_threshold", P.rr_threshold);
        P.rr_cont_prob = json::float_or(r, "rr_cont_prob", P.rr_cont_prob);
        P.state_count = json::int_or(r, "state_count", P.state_count);
        P.albedo = json::bool_or(r, "albedo", P.albedo);
        P.normal = json::bool_or(r, "normal", P.normal);
        if(P.spp <= 0 || P.state_count <= 0)
            throw std::runtime_error("spp and state_count must be positive");
        if(auto f = r->find("filter"))
        {
            const std::string ft = json::as_string(f->child("type"));
            if(ft == "box")
                P.filter = FILTER_BOX;
            else if(ft == "gaussian")
            {
                P.filter = FILTER_GAUSSIAN;
                P.filter_radius = json::float_or(f, "radius", 1.3f);
                P.filter_alpha = json::float_or(f, "alpha", 1.6f);
            }
            else
                throw std::runtime_error("unsupported filter type '" + ft + "'");
        }
        if(auto s = r->find("sampler"))
        {
            const std::string st = s->is_group() ? json::as_string(s->child("type")) : json::as_string(s);
            if(st == "independent")
                P.sampler = SAMPLER_INDEPENDENT;
            else if(st == "halton")
                P.sampler = SAMPLER_HALTON;
            else
                throw std::runtime_error("unsupported sampler type '" + st + "'");
        }
    }

    // scene entities (factory/btrc/factory/scene.cpp:9-55)
    NodeP scene = root->child("scene");
    NodeP ents = scene->child("entities");
    if(!ents->is_array())
        throw std::runtime_error("entity array expected");

    std::map<const json::Node *, int> geo_pool, mat_pool;
    MediumBuilder mb;
    mb.scene_dir = scene_dir;
    S.textures.scene_dir = scene_dir;
    struct PendingInstance { int geo, mat, light; int inner, outer; Transform xf; V3 intensity; };
    std::vector<PendingInstance> pend;
    for(auto &e : ents->elems)
    {
        if(!e->is_group())
            throw std::runtime_error("entity group expected");
        PendingInstance pi{};
        NodeP gn = e->child("geometry");
        auto git = geo_pool.find(gn.get());
        if(git == geo_pool.end())
        {
            const std::string gt = json::as_string(gn->child("type"));
            if(gt == "triangle_mesh")
            {
                const std::string fn = resolve_path(json::as_string(gn->child("filename")), scene_dir);
                S.geometries.push_back(load_obj(fn, json::bool_or(gn, "transform_to_unit_cube", false)));
            }
            else
                S.geometries.push_back(procedural_geometry(gt, json::int_or(gn, "subdivisions", 3)));
            pi.geo = static_cast<int>(S.geometries.size()) - 1;
            geo_pool[gn.get()] = pi.geo;
        }
        else
            pi.geo = git->second;
        NodeP mn = e->child("material");
        auto mit = mat_pool.find(mn.get());
        if(mit == mat_pool.end())
        {
            S.materials.push_back(make_material(mn, S.textures, S.material_tex));
            pi.mat = static_cast<int>(S.materials.size()) - 1;
            mat_pool[mn.get()] = pi.mat;
        }
        else
            pi.mat = mit->second;
        if(auto tn = e->find("local_to_world"))
            pi.xf = parse_transform(tn);
        pi.inner = e->find("inner_medium") ? mb.create(e->find("inner_medium")) : -1;
        pi.outer = e->find("outer_medium") ? mb.create(e->find("outer_medium")) : -1;
        pi.light = -1;
        if(auto ln = e->find("light"))
        {
            const std::string lt = json::as_string(ln->child("type"));
            if(lt != "mesh_light")
                throw std::runtime_error("area light expected");
            pi.light = 1;
            pi.intensity = json::as_spectrum(ln->child("intensity"));
        }
        pend.push_back(pi);
    }
    if(auto vols = scene->find("volumes"))
    {
        // factory/btrc/factory/scene.cpp:57-79
        if(!vols->is_array())
            throw std::runtime_error("'volumes' is not an array node");
        std::vector<VolumePrim> prims;
        for(size_t i = 0; i < vols->elems.size(); ++i)
            prims.push_back(make_volume(vols->elems[i], static_cast<int>(i), scene_dir, S.volume_grids));
        build_volume_bvh(prims, S.volumes, S.volume_nodes);
    }
    if(auto en = scene->find("envir_light"))
    {
        const std::string et = json::as_string(en->child("type"));
        if(et == "gradient_sky")
        {
            S.env.type = ENV_GRADIENT_SKY;
            const V3 up = normalize(json::as_vec3(en->child("up")));
            const V3 lo = json::as_spectrum(en->child("lower"));
            const V3 hi = json::as_spectrum(en->child("upper"));
            S.env.lower[0] = lo.x; S.env.lower[1] = lo.y; S.env.lower[2] = lo.z;
            S.env.upper[0] = hi.x; S.env.upper[1] = hi.y; S.env.upper[2] = hi.z;
            S.env.up[0] = up.x; S.env.up[1] = up.y; S.env.up[2] = up.z;
        }
        else if(et == "ibl")
        {
            // IBLCreator (builtin/btrc/builtin/light/ibl.cpp:80-91)
            S.env.type = ENV_IBL;
            V3 c;
            int prog = compile_texture2d(S.textures, en->child("tex"), c);
            if(prog < 0)
            {
                TexInstr ins{};
                ins.op = TEXOP_CONST;
                ins.a[0] = c.x; ins.a[1] = c.y; ins.a[2] = c.z;
                TexInstr end{};
                end.op = TEXOP_END;
                prog = static_cast<int>(S.textures.instr.size());
                S.textures.instr.push_back(ins);
                S.textures.instr.push_back(end);
            }
            S.env.prog = prog;
            const V3 up = en->find("up") ? json::as_vec3(en->child("up")) : V3(0, 0, 1);
            const Frame f = Frame::from_z(up);
            S.env.frame_x[0] = f.x.x; S.env.frame_x[1] = f.x.y; S.env.frame_x[2] = f.x.z;
            S.env.frame_y[0] = f.y.x; S.env.frame_y[1] = f.y.y; S.env.frame_y[2] = f.y.z;
            S.env.up[0] = f.z.x; S.env.up[1] = f.z.y; S.env.up[2] = f.z.z;
            S.env.lut_w = json::int_or(en, "lut_width", 400);
            S.env.lut_h = json::int_or(en, "lut_height", 200);
            if(S.env.lut_w <= 0 || S.env.lut_h <= 0 || S.env.lut_w > 8192 || S.env.lut_h > 8192)
                throw std::runtime_error("ibl lut size out of range");
            build_env_sampler(S.textures, prog, S.env.lut_w, S.env.lut_h, S.env_probs, S.env_alias);
        }
        else
            throw std::runtime_error("unsupported environment light '" + et + "'");
    }

    // medium id table (core/btrc/core/scene.cpp:136-161): media sorted by priority
    // descending (stable), the volume-primitive medium (vacuum here) last; entities
    // without a medium refer to it.
    {
        std::vector<int> order(mb.media.size());
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            return mb.media[a].priority > mb.media[b].priority;
        });
        std::vector<int> remap(mb.media.size());
        for(size_t i = 0; i < order.size(); ++i)
        {
            remap[order[i]] = static_cast<int>(i);
            S.media.push_back(std::move(mb.media[order[i]]));
        }
        HostMedium vac{};
        vac.dev.type = S.volumes.empty() ? MED_VACUUM : MED_VOLUMES;
        vac.dev.priority = -(1 << 30);
        S.media.push_back(vac);
        S.vacuum_medium = static_cast<int>(S.media.size()) - 1;
        for(auto &pi : pend)
        {
            pi.inner = pi.inner < 0 ? S.vacuum_medium : remap[pi.inner];
            pi.outer = pi.outer < 0 ? S.vacuum_medium : remap[pi.outer];
        }
    }

    // instances and lights in entity order (core/btrc/core/scene.cpp:92-101, 163-190)
    int next_light = 0;
    for(size_t i = 0; i < pend.size(); ++i)
    {
        auto &pi = pend[i];
        Instance inst{};
        pi.xf.to_affine(inst.l2w, inst.w2l);
        inst.geometry = pi.geo;
        inst.material = pi.mat;
        inst.light = -1;
        inst.media = static_cast<uint32_t>(pi.inner) | (static_cast<uint32_t>(pi.outer) << 16);
        if(pi.light >= 0)
        {
            inst.light = next_light++;
            AreaLight L{};
            L.instance = static_cast<int>(i);
            L.geometry = pi.geo;
            // builtin/btrc/builtin/light/mesh_light.cpp:10-15
            L.scale = length(pi.xf.point(V3(1, 0, 0)) - pi.xf.point(V3(0, 0, 0)));
            L.intensity[0] = pi.intensity.x; L.intensity[1] = pi.intensity.y; L.intensity[2] = pi.intensity.z;
            S.area_lights.push_back(L);
        }
        S.instances.push_back(inst);
        S.instance_xf.push_back(pi.xf);
        S.triangle_count += S.geometries[pi.geo].area.size();
    }

    // world bounds (core/btrc/core/scene.cpp:224-236) from transformed geometry boxes
    S.world_min = V3(MAX_FLOAT);
    S.world_max = V3(-MAX_FLOAT);
    for(size_t i = 0; i < S.instances.size(); ++i)
    {
        const HostGeometry &g = S.geometries[S.instances[i].geometry];
        if(g.area.empty())
            continue;
        for(int c = 0; c < 8; ++c)
        {
            const V3 p((c & 1) ? g.bmax.x : g.bmin.x, (c & 2) ? g.bmax.y : g.bmin.y, (c & 4) ? g.bmax.z : g.bmin.z);
            const V3 w = S.instance_xf[i].point(p);
            S.world_min = vmin(S.world_min, w);
            S.world_max = vmax(S.world_max, w);
        }
    }
    // volume boxes join the world bounds (core/btrc/core/scene.cpp:233-237)
    for(const VolumePrim &v : S.volumes)
    {
        const V3 lo = volume_box_lower(v), hi = volume_box_upper(v);
        S.world_min = vmin(S.world_min, lo);
        S.world_max = vmax(S.world_max, hi);
    }
    if(S.world_min.x > S.world_max.x)
    {
        S.world_min = V3(0);
        S.world_max = V3(0);
    }
    return S;
}

} // namespace bt
