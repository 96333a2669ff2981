#include "bvh.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <stdexcept>
#include <thread>

namespace bt {

namespace {

constexpr int NUM_BINS = 32;
constexpr uint32_t MAX_LEAF = 3;      // a wide-node leaf child holds up to 3 triangles
constexpr int MAX_BINARY_DEPTH = 64;  // deeper nodes fall back to median splits
constexpr double COST_TRAVERSE = 1.0;
constexpr double COST_INTERSECT = 1.0;
// SAH weights of the wide collapse: a wide-node test (8 child boxes) against one triangle
// test, in the traversal kernel's instruction counts
constexpr float WIDE_COST_NODE = 1.0f;
constexpr float WIDE_COST_TRI = 0.4f;

// parallel granularity: ranges above PAR_RANGE are binned and partitioned by several
// threads at once; subtrees above TASK_RANGE become tasks of their own
constexpr uint32_t PAR_RANGE = 1u << 17;
constexpr uint32_t TASK_RANGE = 1u << 12;
constexpr size_t PAR_CHUNK = 1u << 15;
// ranges up to SMALL_RANGE choose their plane without bin tables
constexpr uint32_t SMALL_RANGE = 24;

struct Box
{
    float lo[3] = { MAX_FLOAT, MAX_FLOAT, MAX_FLOAT };
    float hi[3] = { -MAX_FLOAT, -MAX_FLOAT, -MAX_FLOAT };
    void grow(const float *l, const float *h)
    {
        for(int k = 0; k < 3; ++k)
        {
            lo[k] = std::min(lo[k], l[k]);
            hi[k] = std::max(hi[k], h[k]);
        }
    }
    void grow(const Box &b) { grow(b.lo, b.hi); }
    double area() const
    {
        if(lo[0] > hi[0])
            return 0;
        const double dx = (double)hi[0] - lo[0], dy = (double)hi[1] - lo[1], dz = (double)hi[2] - lo[2];
        return 2.0 * (dx * dy + dy * dz + dz * dx);
    }
};

// one triangle reference: its bounds and index (32 bytes, moved by the partitions)
struct Ref
{
    float lo[3];
    uint32_t id;
    float hi[3];
    uint32_t pad;
    float cen(int a) const { return 0.5f * (lo[a] + hi[a]); }
};

// binary node; plain data, so that the node array is not touched before the build
// writes it
struct BNode
{
    float lo[3], hi[3];
    int32_t left, right;  // left < 0: leaf
    uint32_t first, count;
    Box bbox() const
    {
        Box b;
        b.grow(lo, hi);
        return b;
    }
    void set_box(const Box &b)
    {
        for(int k = 0; k < 3; ++k)
        {
            lo[k] = b.lo[k];
            hi[k] = b.hi[k];
        }
    }
};

// bounds of a range: the boxes and the centroids
struct Bounds
{
    Box box, cbox;
    void add(const Ref &r)
    {
        box.grow(r.lo, r.hi);
        const float c[3] = { r.cen(0), r.cen(1), r.cen(2) };
        cbox.grow(c, c);
    }
    void add(const Bounds &o)
    {
        box.grow(o.box);
        cbox.grow(o.cbox);
    }
};

struct Bins
{
    Box box[3][NUM_BINS];
    uint32_t cnt[3][NUM_BINS] = {};
    void add(const Bins &o)
    {
        for(int a = 0; a < 3; ++a)
            for(int k = 0; k < NUM_BINS; ++k)
            {
                box[a][k].grow(o.box[a][k]);
                cnt[a][k] += o.cnt[a][k];
            }
    }
};

// Binned SAH over a triangle set (FP64 costs), built top-down with fork-join tasks; each
// node's 8-wide collapse cost table is filled once both children are done.
class Builder
{
public:
    Builder(const std::vector<TriRec> &t, TaskPool &pool) : tris_(t), pool_(pool)
    {
        const size_t n = t.size();
        refs_.reset(new Ref[n]);
        tmp_.reset(new Ref[n]);
        const size_t cap = std::max<size_t>(1, 2 * n);
        nodes_.reset(new BNode[cap]);
        cost_.reset(new float[cap * 8]);
        split_.reset(new uint8_t[cap * 8]);
        split8_.reset(new uint8_t[cap]);
        as_leaf_.reset(new uint8_t[cap]);
        ntri_.reset(new uint32_t[cap]);
    }

    void run()
    {
        const size_t n = tris_.size();
        std::vector<Bounds> part(static_cast<size_t>(pool_.threads()) * 4 + 1);
        std::atomic<int> slot{ 0 };
        pool_.parallel_for(n, PAR_CHUNK, [&](size_t b, size_t e) {
            Bounds acc;
            for(size_t i = b; i < e; ++i)
            {
                const TriRec &r = tris_[i];
                Ref &f = refs_[i];
                f.lo[0] = std::min(std::min(r.v0x, r.v1x), r.v2x);
                f.lo[1] = std::min(std::min(r.v0y, r.v1y), r.v2y);
                f.lo[2] = std::min(std::min(r.v0z, r.v1z), r.v2z);
                f.hi[0] = std::max(std::max(r.v0x, r.v1x), r.v2x);
                f.hi[1] = std::max(std::max(r.v0y, r.v1y), r.v2y);
                f.hi[2] = std::max(std::max(r.v0z, r.v1z), r.v2z);
                f.id = static_cast<uint32_t>(i);
                f.pad = 0;
                acc.add(f);
            }
            part[slot.fetch_add(1)] = acc;
        });
        Bounds root;
        for(int k = 0; k < slot.load(); ++k)
            root.add(part[k]);
        node_count_ = 1;
        build(0, 0, static_cast<uint32_t>(n), root, 0);
    }

    int node_count() const { return node_count_.load(); }

    // outputs
    std::unique_ptr<Ref[]> refs_;
    std::unique_ptr<BNode[]> nodes_;
    std::unique_ptr<float[]> cost_;
    std::unique_ptr<uint8_t[]> split_;    // [n][i-1], i >= 2: left share k, 0: same as i - 1
    std::unique_ptr<uint8_t[]> split8_;   // left share of the 8-slot distribution
    std::unique_ptr<uint8_t[]> as_leaf_;
    std::unique_ptr<uint32_t[]> ntri_;

private:
    const std::vector<TriRec> &tris_;
    TaskPool &pool_;
    std::unique_ptr<Ref[]> tmp_;
    std::atomic<int> node_count_{ 0 };

    static int bin_of(float c, float cmin, double scale)
    {
        const int bi = static_cast<int>(((double)c - cmin) * scale);
        return std::min(NUM_BINS - 1, std::max(0, bi));
    }

    void bin_range(uint32_t b, uint32_t e, const Box &cbox, const double *scale, Bins &out) const
    {
        for(uint32_t i = b; i < e; ++i)
        {
            const Ref &r = refs_[i];
            for(int a = 0; a < 3; ++a)
            {
                if(!(scale[a] > 0))
                    continue;
                const int bi = bin_of(r.cen(a), cbox.lo[a], scale[a]);
                out.box[a][bi].grow(r.lo, r.hi);
                ++out.cnt[a][bi];
            }
        }
    }

    // Best SAH plane from the bins of each axis. The cost is the same for every plane
    // between two occupied bins and the sweep keeps the first plane of least cost, so it
    // visits only the plane after each occupied bin.
    static void sweep_bins(const Bins &bins, const double *scale, double &best_cost, int &best_axis, int &best_bin)
    {
        for(int axis = 0; axis < 3; ++axis)
        {
            if(!(scale[axis] > 0))
                continue;
            int occ[NUM_BINS];
            int m = 0;
            for(int k = 0; k < NUM_BINS; ++k)
                if(bins.cnt[axis][k])
                    occ[m++] = k;
            if(m < 2)
                continue;
            double right_area[NUM_BINS];
            uint32_t right_cnt[NUM_BINS];
            Box acc;
            uint32_t ac = 0;
            for(int j = m - 1; j > 0; --j)
            {
                acc.grow(bins.box[axis][occ[j]]);
                ac += bins.cnt[axis][occ[j]];
                right_area[j] = acc.area();
                right_cnt[j] = ac;
            }
            Box lacc;
            uint32_t lc = 0;
            for(int j = 0; j < m - 1; ++j)
            {
                lacc.grow(bins.box[axis][occ[j]]);
                lc += bins.cnt[axis][occ[j]];
                const double c = lacc.area() * lc + right_area[j + 1] * right_cnt[j + 1];
                if(c < best_cost)
                {
                    best_cost = c;
                    best_axis = axis;
                    best_bin = occ[j];
                }
            }
        }
    }

    // The same choice for a handful of references without bin tables: per axis, the
    // references ordered by bin index form the occupied bins directly.
    void sweep_small(uint32_t b, uint32_t e, const Box &cbox, const double *scale, double &best_cost, int &best_axis,
                     int &best_bin) const
    {
        const uint32_t n = e - b;
        for(int axis = 0; axis < 3; ++axis)
        {
            if(!(scale[axis] > 0))
                continue;
            int bin[SMALL_RANGE];
            uint32_t ord[SMALL_RANGE];
            for(uint32_t i = 0; i < n; ++i)
            {
                bin[i] = bin_of(refs_[b + i].cen(axis), cbox.lo[axis], scale[axis]);
                uint32_t j = i;  // insertion by bin index
                while(j > 0 && bin[ord[j - 1]] > bin[i])
                {
                    ord[j] = ord[j - 1];
                    --j;
                }
                ord[j] = i;
            }
            double right_area[SMALL_RANGE];
            Box acc;
            for(uint32_t j = n; j-- > 1;)
            {
                const Ref &r = refs_[b + ord[j]];
                acc.grow(r.lo, r.hi);
                right_area[j] = acc.area();
            }
            Box lacc;
            for(uint32_t j = 0; j + 1 < n; ++j)
            {
                const Ref &r = refs_[b + ord[j]];
                lacc.grow(r.lo, r.hi);
                if(bin[ord[j]] == bin[ord[j + 1]])
                    continue;  // a plane lies only after the last reference of a bin
                const double c = lacc.area() * static_cast<double>(j + 1) + right_area[j + 1] * static_cast<double>(n - j - 1);
                if(c < best_cost)
                {
                    best_cost = c;
                    best_axis = axis;
                    best_bin = bin[ord[j]];
                }
            }
        }
    }

    void make_leaf(int ni, uint32_t b, uint32_t e)
    {
        BNode &nd = nodes_[ni];
        nd.left = nd.right = -1;
        nd.first = b;
        nd.count = e - b;
        const float A = static_cast<float>(nd.bbox().area());
        float *c = &cost_[static_cast<size_t>(ni) * 8];
        for(int i = 0; i < 8; ++i)
        {
            c[i] = A * WIDE_COST_TRI * static_cast<float>(nd.count);
            split_[static_cast<size_t>(ni) * 8 + i] = 0;
        }
        split8_[ni] = 0;
        as_leaf_[ni] = 1;
        ntri_[ni] = nd.count;
    }

    // partition [b, e) so that refs with pred true come first; returns the split point
    // and the bounds of both sides. Large ranges: per-chunk counts, then a parallel
    // scatter through the spare buffer (stable); small ranges: in place.
    template<class Pred>
    uint32_t partition(uint32_t b, uint32_t e, Pred &&pred, Bounds &lb, Bounds &rb)
    {
        const uint32_t count = e - b;
        if(count <= PAR_RANGE)
        {
            Ref *first = &refs_[b], *last = &refs_[b] + count;
            Ref *mid = std::partition(first, last, pred);
            for(Ref *p = first; p < mid; ++p)
                lb.add(*p);
            for(Ref *p = mid; p < last; ++p)
                rb.add(*p);
            return b + static_cast<uint32_t>(mid - first);
        }
        const size_t chunk = PAR_CHUNK;
        const size_t nch = (count + chunk - 1) / chunk;
        std::vector<uint32_t> nleft(nch);
        std::vector<Bounds> lbs(nch), rbs(nch);
        pool_.parallel_for(nch, 1, [&](size_t c0, size_t c1) {
            for(size_t c = c0; c < c1; ++c)
            {
                const uint32_t s = b + static_cast<uint32_t>(c * chunk);
                const uint32_t t = std::min(e, static_cast<uint32_t>(s + chunk));
                uint32_t k = 0;
                for(uint32_t i = s; i < t; ++i)
                    if(pred(refs_[i]))
                    {
                        ++k;
                        lbs[c].add(refs_[i]);
                    }
                    else
                        rbs[c].add(refs_[i]);
                nleft[c] = k;
            }
        });
        std::vector<uint32_t> loff(nch), roff(nch);
        uint32_t total_left = 0;
        for(size_t c = 0; c < nch; ++c)
        {
            loff[c] = total_left;
            total_left += nleft[c];
        }
        uint32_t r = total_left;
        for(size_t c = 0; c < nch; ++c)
        {
            roff[c] = r;
            const uint32_t s = static_cast<uint32_t>(c * chunk);
            r += std::min<uint32_t>(count - s, static_cast<uint32_t>(chunk)) - nleft[c];
            lb.add(lbs[c]);
            rb.add(rbs[c]);
        }
        pool_.parallel_for(nch, 1, [&](size_t c0, size_t c1) {
            for(size_t c = c0; c < c1; ++c)
            {
                const uint32_t s = b + static_cast<uint32_t>(c * chunk);
                const uint32_t t = std::min(e, static_cast<uint32_t>(s + chunk));
                uint32_t li = b + loff[c], ri = b + roff[c];
                for(uint32_t i = s; i < t; ++i)
                    tmp_[pred(refs_[i]) ? li++ : ri++] = refs_[i];
            }
        });
        pool_.parallel_for(count, PAR_CHUNK, [&](size_t s, size_t t) {
            std::memcpy(&refs_[b + s], &tmp_[b + s], (t - s) * sizeof(Ref));
        });
        return b + total_left;
    }

    void build(int ni, uint32_t b, uint32_t e, const Bounds &bounds, int depth)
    {
        BNode &nd = nodes_[ni];
        nd.set_box(bounds.box);
        const Box &cbox = bounds.cbox;
        const uint32_t count = e - b;
        if(count <= 1)
        {
            make_leaf(ni, b, e);
            return;
        }

        uint32_t mid = 0;
        bool split_found = false;
        Bounds lb, rb;
        if(depth < MAX_BINARY_DEPTH)
        {
            double scale[3];
            for(int a = 0; a < 3; ++a)
            {
                const float cmin = cbox.lo[a], cmax = cbox.hi[a];
                scale[a] = cmax > cmin ? NUM_BINS / ((double)cmax - cmin) : 0.0;
            }
            double best_cost = std::numeric_limits<double>::infinity();
            int best_axis = -1, best_bin = -1;
            if(count <= SMALL_RANGE)
                sweep_small(b, e, cbox, scale, best_cost, best_axis, best_bin);
            else
            {
                Bins bins;
                if(count > PAR_RANGE)
                {
                    const size_t nch = (count + PAR_CHUNK - 1) / PAR_CHUNK;
                    std::vector<Bins> part(nch);
                    pool_.parallel_for(nch, 1, [&](size_t c0, size_t c1) {
                        for(size_t c = c0; c < c1; ++c)
                        {
                            const uint32_t s = b + static_cast<uint32_t>(c * PAR_CHUNK);
                            bin_range(s, std::min(e, static_cast<uint32_t>(s + PAR_CHUNK)), cbox, scale, part[c]);
                        }
                    });
                    for(auto &p : part)
                        bins.add(p);
                }
                else
                    bin_range(b, e, cbox, scale, bins);
                sweep_bins(bins, scale, best_cost, best_axis, best_bin);
            }
            if(best_axis >= 0)
            {
                const double parent_area = std::max(nd.bbox().area(), 1e-300);
                const double split_cost = COST_TRAVERSE + COST_INTERSECT * best_cost / parent_area;
                const double leaf_cost = COST_INTERSECT * count;
                if(count <= MAX_LEAF && leaf_cost <= split_cost)
                {
                    make_leaf(ni, b, e);
                    return;
                }
                const float cmin = cbox.lo[best_axis];
                const double sc = scale[best_axis];
                const int ax = best_axis, bb = best_bin;
                mid = partition(b, e, [cmin, sc, ax, bb](const Ref &r) { return bin_of(r.cen(ax), cmin, sc) <= bb; },
                                lb, rb);
                split_found = mid > b && mid < e;
            }
        }
        if(!split_found)
        {
            if(count <= MAX_LEAF)
            {
                make_leaf(ni, b, e);
                return;
            }
            // identical centroids or too deep: split the index range in half along the
            // widest centroid axis
            int axis = 0;
            float ext = -1;
            for(int k = 0; k < 3; ++k)
                if(cbox.hi[k] - cbox.lo[k] > ext)
                {
                    ext = cbox.hi[k] - cbox.lo[k];
                    axis = k;
                }
            mid = b + count / 2;
            std::nth_element(&refs_[b], &refs_[mid], &refs_[b] + count, [axis](const Ref &x, const Ref &y) {
                return x.cen(axis) < y.cen(axis);
            });
            lb = Bounds();
            rb = Bounds();
            for(uint32_t i = b; i < mid; ++i)
                lb.add(refs_[i]);
            for(uint32_t i = mid; i < e; ++i)
                rb.add(refs_[i]);
        }

        const int l = node_count_.fetch_add(2);
        nd.left = l;
        nd.right = l + 1;
        nd.count = 0;
        if(count > TASK_RANGE)
        {
            TaskPool::Group g;
            pool_.run(g, [this, l, b, mid, lb, depth] { build(l, b, mid, lb, depth + 1); });
            build(l + 1, mid, e, rb, depth + 1);
            pool_.wait(g);
        }
        else
        {
            build(l, b, mid, lb, depth + 1);
            build(l + 1, mid, e, rb, depth + 1);
        }
        collapse_costs(ni);
    }

    // Wide collapse by dynamic programming over the binary tree (Ylitie, Karras and
    // Laine, "Efficient incoherent ray traversal on GPUs through compressed wide BVHs",
    // HPG 2017, section 3): C(n, i) is the least SAH cost of the subtree of n spread
    // over at most i child slots of a wide node; one slot holds either a leaf of <= 3
    // triangles or a wide node whose 8 slots hold the subtree.
    void collapse_costs(int q)
    {
        const BNode &nd = nodes_[q];
        const float A = static_cast<float>(nd.bbox().area());
        const float INF = std::numeric_limits<float>::infinity();
        float *c = &cost_[static_cast<size_t>(q) * 8];
        uint8_t *sp = &split_[static_cast<size_t>(q) * 8];
        ntri_[q] = ntri_[nd.left] + ntri_[nd.right];
        const float *cl = &cost_[static_cast<size_t>(nd.left) * 8], *cr = &cost_[static_cast<size_t>(nd.right) * 8];
        float dist[9];
        uint8_t arg[9] = {};
        for(int j = 2; j <= 8; ++j)
        {
            dist[j] = INF;
            for(int k = 1; k < j; ++k)
            {
                const float v = cl[k - 1] + cr[j - k - 1];
                if(v < dist[j])
                {
                    dist[j] = v;
                    arg[j] = static_cast<uint8_t>(k);
                }
            }
        }
        split8_[q] = arg[8];
        const float c_internal = A * WIDE_COST_NODE + dist[8];
        const float c_leaf = ntri_[q] <= MAX_LEAF ? A * WIDE_COST_TRI * static_cast<float>(ntri_[q]) : INF;
        as_leaf_[q] = c_leaf <= c_internal ? 1 : 0;
        c[0] = std::min(c_leaf, c_internal);
        sp[0] = 0;
        for(int i = 2; i <= 8; ++i)
        {
            if(dist[i] < c[i - 2])
            {
                c[i - 1] = dist[i];
                sp[i - 1] = arg[i];
            }
            else
            {
                c[i - 1] = c[i - 2];
                sp[i - 1] = 0;
            }
        }
    }
};

// Smallest e with 255 * 2^e >= extent, clamped so that 2^e is a normal float.
int quant_exponent(double extent)
{
    if(!(extent > 0))
        return -126;
    int e = static_cast<int>(std::ceil(std::log2(extent / 255.0)));
    while(std::ldexp(255.0, e) < extent)
        ++e;
    while(e > -126 && std::ldexp(255.0, e - 1) >= extent)
        --e;
    return std::max(-126, std::min(127, e));
}

// the children of one wide node: binary subtrees in slots, and what they hold
struct WideKids
{
    int n = 0;
    int kid[8];          // binary node of each child
    int kid_in_slot[8];  // child index in slot s, or -1
    uint32_t n_internal = 0, n_tris = 0;
};

} // namespace

CWBVH build_cwbvh(const std::vector<TriRec> &tris, TaskPool &pool)
{
    CWBVH out;
    if(tris.empty())
        return out;

    Builder bb(tris, pool);
    bb.run();
    out.binary_nodes = bb.node_count();
    const BNode *bn = bb.nodes_.get();
    const uint8_t *split = bb.split_.get();
    const uint8_t *split8 = bb.split8_.get();
    const uint8_t *as_leaf = bb.as_leaf_.get();
    const uint32_t *ntri = bb.ntri_.get();
    const Ref *refs = bb.refs_.get();

    // the slots a subtree takes when it may use up to i of them
    auto expand = [&](auto &&self, int m, int i, WideKids &w) -> void {
        while(i >= 2 && split[static_cast<size_t>(m) * 8 + i - 1] == 0)
            --i;
        if(i == 1)
        {
            w.kid[w.n++] = m;
            return;
        }
        const int k = split[static_cast<size_t>(m) * 8 + i - 1];
        self(self, bn[m].left, k, w);
        self(self, bn[m].right, i - k, w);
    };
    // triangles (binary-leaf ranges) of a subtree kept as one leaf slot, in order
    auto leaf_tris = [&](int m, TriRec *dst) {
        int st[2 * MAX_BINARY_DEPTH + 8];
        int sp = 0;
        st[sp++] = m;
        uint32_t k = 0;
        while(sp > 0)
        {
            const int x = st[--sp];
            if(bn[x].left < 0)
            {
                for(uint32_t t = 0; t < bn[x].count; ++t)
                    dst[k++] = tris[refs[bn[x].first + t].id];
            }
            else
            {
                st[sp++] = bn[x].right;
                st[sp++] = bn[x].left;
            }
        }
        return k;
    };
    auto make_kids = [&](int m, WideKids &w) {
        w = WideKids{};
        const BNode &root = bn[m];
        if(root.left < 0)
            w.kid[w.n++] = m;
        else
        {
            const int k = split8[m];
            expand(expand, root.left, k, w);
            expand(expand, root.right, 8 - k, w);
        }
        // slot assignment: slot s prefers children far along (s&1?+x:-x, s&2?+y:-y,
        // s&4?+z:-z); the traversal visits slot == ray octant first
        Box nbox;
        for(int k = 0; k < w.n; ++k)
            nbox.grow(bn[w.kid[k]].lo, bn[w.kid[k]].hi);
        double pc[3];
        for(int a = 0; a < 3; ++a)
            pc[a] = 0.5 * ((double)nbox.lo[a] + nbox.hi[a]);
        for(int s = 0; s < 8; ++s)
            w.kid_in_slot[s] = -1;
        double cost[8][8];
        for(int k = 0; k < w.n; ++k)
        {
            const BNode &cb = bn[w.kid[k]];
            double cc[3];
            for(int a = 0; a < 3; ++a)
                cc[a] = 0.5 * ((double)cb.lo[a] + cb.hi[a]) - pc[a];
            for(int s = 0; s < 8; ++s)
                cost[k][s] = ((s & 1) ? cc[0] : -cc[0]) + ((s & 2) ? cc[1] : -cc[1]) + ((s & 4) ? cc[2] : -cc[2]);
        }
        bool kid_done[8] = {};
        for(int round = 0; round < w.n; ++round)
        {
            int bk = -1, bs = -1;
            double bc = -std::numeric_limits<double>::infinity();
            for(int k = 0; k < w.n; ++k)
            {
                if(kid_done[k])
                    continue;
                for(int s = 0; s < 8; ++s)
                    if(w.kid_in_slot[s] < 0 && cost[k][s] > bc)
                    {
                        bc = cost[k][s];
                        bk = k;
                        bs = s;
                    }
            }
            kid_done[bk] = true;
            w.kid_in_slot[bs] = bk;
        }
        for(int k = 0; k < w.n; ++k)
        {
            if(as_leaf[w.kid[k]])
                w.n_tris += ntri[w.kid[k]];
            else
                ++w.n_internal;
        }
    };

    // emit level by level: the wide nodes of a level are consecutive, each node's
    // internal children are consecutive in the next level, and leaf triangles follow
    // node order (a per-level prefix sum gives every node its child and triangle base)
    out.nodes.resize(1);
    out.tris.resize(tris.size());
    std::vector<int> level{ 0 };  // binary node of each wide node of the level
    uint32_t level_base = 0;      // wide-node index of the level's first node
    uint32_t tri_cursor = 0;
    std::vector<WideKids> kids;
    std::vector<uint32_t> child_base, tri_base;
    while(!level.empty())
    {
        ++out.depth;
        const size_t n = level.size();
        kids.resize(n);
        pool.parallel_for(n, 256, [&](size_t b, size_t e) {
            for(size_t i = b; i < e; ++i)
                make_kids(level[i], kids[i]);
        });
        child_base.resize(n);
        tri_base.resize(n);
        const uint32_t next_base = level_base + static_cast<uint32_t>(n);
        uint32_t nc = next_base, tc = tri_cursor;
        for(size_t i = 0; i < n; ++i)
        {
            child_base[i] = nc;
            tri_base[i] = tc;
            nc += kids[i].n_internal;
            tc += kids[i].n_tris;
        }
        if(tc > tris.size())
            throw std::runtime_error("BVH collapse lost track of its triangles");
        out.nodes.resize(nc);
        std::vector<int> next(nc - next_base);
        pool.parallel_for(n, 256, [&](size_t b, size_t e) {
            for(size_t i = b; i < e; ++i)
            {
                const WideKids &w = kids[i];
                Box nbox;
                for(int k = 0; k < w.n; ++k)
                    nbox.grow(bn[w.kid[k]].lo, bn[w.kid[k]].hi);
                CWNode node{};
                node.px = nbox.lo[0];
                node.py = nbox.lo[1];
                node.pz = nbox.lo[2];
                int ex[3];
                for(int a = 0; a < 3; ++a)
                    ex[a] = quant_exponent((double)nbox.hi[a] - (double)nbox.lo[a]);
                node.ex = static_cast<uint8_t>(ex[0] + 127);
                node.ey = static_cast<uint8_t>(ex[1] + 127);
                node.ez = static_cast<uint8_t>(ex[2] + 127);
                node.child_base = child_base[i];
                node.tri_base = tri_base[i];
                node.imask = 0;
                uint32_t tri_off = 0;
                int next_internal = 0;
                for(int s = 0; s < 8; ++s)
                {
                    const int k = w.kid_in_slot[s];
                    if(k < 0)
                    {
                        node.meta[s] = 0;
                        continue;
                    }
                    const int m = w.kid[k];
                    const BNode &c = bn[m];
                    // quantise (exact in double: power-of-two scale)
                    const double org[3] = { (double)node.px, (double)node.py, (double)node.pz };
                    uint8_t ql[3], qh[3];
                    for(int a = 0; a < 3; ++a)
                    {
                        const double sc = std::ldexp(1.0, ex[a]);
                        double l = std::floor(((double)c.lo[a] - org[a]) / sc);
                        double h = std::ceil(((double)c.hi[a] - org[a]) / sc);
                        l = std::max(0.0, std::min(255.0, l));
                        h = std::max(0.0, std::min(255.0, h));
                        ql[a] = static_cast<uint8_t>(l);
                        qh[a] = static_cast<uint8_t>(h);
                    }
                    node.qlo_x[s] = ql[0]; node.qlo_y[s] = ql[1]; node.qlo_z[s] = ql[2];
                    node.qhi_x[s] = qh[0]; node.qhi_y[s] = qh[1]; node.qhi_z[s] = qh[2];
                    if(!as_leaf[m])
                    {
                        node.imask |= static_cast<uint8_t>(1u << s);
                        node.meta[s] = static_cast<uint8_t>((1u << 5) | (24u + s));
                        next[child_base[i] - next_base + next_internal++] = m;
                    }
                    else
                    {
                        static const uint8_t unary[4] = { 0, 1, 3, 7 };
                        const uint32_t cnt = leaf_tris(m, &out.tris[tri_base[i] + tri_off]);
                        node.meta[s] = static_cast<uint8_t>((unary[cnt] << 5) | tri_off);
                        tri_off += cnt;
                    }
                }
                out.nodes[level_base + i] = node;
            }
        });
        level.swap(next);
        level_base = next_base;
        tri_cursor = tc;
    }
    if(tri_cursor != tris.size())
        throw std::runtime_error("BVH collapse lost track of its triangles");
    if(out.depth > TRAVERSAL_STACK_SIZE)
        throw std::runtime_error("BVH too deep for the traversal stack (" + std::to_string(out.depth) + " levels)");
    return out;
}

CWBVH build_cwbvh(const std::vector<TriRec> &tris, int threads)
{
    if(threads <= 0)
        threads = std::max(1u, std::thread::hardware_concurrency());
    TaskPool pool(threads);
    return build_cwbvh(tris, pool);
}

} // namespace bt
