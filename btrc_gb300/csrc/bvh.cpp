#include "bvh.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <deque>
#include <limits>
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

struct BNode
{
    Box box;
    int32_t left = -1, right = -1;  // left < 0: leaf
    uint32_t first = 0, count = 0;
};

class BinaryBuilder
{
public:
    BinaryBuilder(const std::vector<TriRec> &t, int threads) : tris_(t), threads_(threads)
    {
        const size_t n = t.size();
        boxes_.resize(n);
        cen_.resize(n * 3);
        idx_.resize(n);
        for(size_t i = 0; i < n; ++i)
        {
            const TriRec &r = t[i];
            Box b;
            const float v0[3] = { r.v0x, r.v0y, r.v0z }, v1[3] = { r.v1x, r.v1y, r.v1z },
                        v2[3] = { r.v2x, r.v2y, r.v2z };
            b.grow(v0, v0);
            b.grow(v1, v1);
            b.grow(v2, v2);
            boxes_[i] = b;
            for(int k = 0; k < 3; ++k)
                cen_[i * 3 + k] = 0.5f * (b.lo[k] + b.hi[k]);
            idx_[i] = static_cast<uint32_t>(i);
        }
        nodes_.resize(std::max<size_t>(1, 2 * n));
    }

    void run()
    {
        node_count_ = 1;
        build(0, 0, static_cast<uint32_t>(tris_.size()), 0);
        nodes_.resize(node_count_.load());
    }

    std::vector<BNode> nodes_;
    std::vector<uint32_t> idx_;

private:
    const std::vector<TriRec> &tris_;
    int threads_;
    std::vector<Box> boxes_;
    std::vector<float> cen_;
    std::atomic<int> node_count_{ 0 };
    std::atomic<int> live_threads_{ 1 };

    void make_leaf(BNode &nd, uint32_t b, uint32_t e)
    {
        nd.left = nd.right = -1;
        nd.first = b;
        nd.count = e - b;
    }

    void build(int ni, uint32_t b, uint32_t e, int depth)
    {
        BNode &nd = nodes_[ni];
        Box box, cbox;
        for(uint32_t i = b; i < e; ++i)
        {
            box.grow(boxes_[idx_[i]]);
            const float *c = &cen_[idx_[i] * 3];
            cbox.grow(c, c);
        }
        nd.box = box;
        const uint32_t count = e - b;
        if(count <= 1)
        {
            make_leaf(nd, b, e);
            return;
        }

        uint32_t mid = 0;
        bool split_found = false;
        if(depth < MAX_BINARY_DEPTH)
        {
            double best_cost = std::numeric_limits<double>::infinity();
            int best_axis = -1, best_bin = -1;
            for(int axis = 0; axis < 3; ++axis)
            {
                const float cmin = cbox.lo[axis], cmax = cbox.hi[axis];
                if(!(cmax > cmin))
                    continue;
                const double scale = NUM_BINS / ((double)cmax - cmin);
                Box bins[NUM_BINS];
                uint32_t cnt[NUM_BINS] = {};
                for(uint32_t i = b; i < e; ++i)
                {
                    const uint32_t p = idx_[i];
                    int bi = static_cast<int>(((double)cen_[p * 3 + axis] - cmin) * scale);
                    bi = std::min(NUM_BINS - 1, std::max(0, bi));
                    bins[bi].grow(boxes_[p]);
                    ++cnt[bi];
                }
                double right_area[NUM_BINS];
                uint32_t right_cnt[NUM_BINS];
                Box acc;
                uint32_t ac = 0;
                for(int k = NUM_BINS - 1; k > 0; --k)
                {
                    acc.grow(bins[k]);
                    ac += cnt[k];
                    right_area[k] = acc.area();
                    right_cnt[k] = ac;
                }
                Box lacc;
                uint32_t lc = 0;
                for(int k = 0; k < NUM_BINS - 1; ++k)
                {
                    lacc.grow(bins[k]);
                    lc += cnt[k];
                    if(lc == 0 || right_cnt[k + 1] == 0)
                        continue;
                    const double c = lacc.area() * lc + right_area[k + 1] * right_cnt[k + 1];
                    if(c < best_cost)
                    {
                        best_cost = c;
                        best_axis = axis;
                        best_bin = k;
                    }
                }
            }
            if(best_axis >= 0)
            {
                const double parent_area = std::max(box.area(), 1e-300);
                const double split_cost = COST_TRAVERSE + COST_INTERSECT * best_cost / parent_area;
                const double leaf_cost = COST_INTERSECT * count;
                if(count <= MAX_LEAF && leaf_cost <= split_cost)
                {
                    make_leaf(nd, b, e);
                    return;
                }
                const float cmin = cbox.lo[best_axis], cmax = cbox.hi[best_axis];
                const double scale = NUM_BINS / ((double)cmax - cmin);
                auto it = std::partition(idx_.begin() + b, idx_.begin() + e, [&](uint32_t p) {
                    int bi = static_cast<int>(((double)cen_[p * 3 + best_axis] - cmin) * scale);
                    bi = std::min(NUM_BINS - 1, std::max(0, bi));
                    return bi <= best_bin;
                });
                mid = static_cast<uint32_t>(it - idx_.begin());
                split_found = mid > b && mid < e;
            }
        }
        if(!split_found)
        {
            if(count <= MAX_LEAF)
            {
                make_leaf(nd, b, e);
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
            std::nth_element(idx_.begin() + b, idx_.begin() + mid, idx_.begin() + e, [&](uint32_t x, uint32_t y) {
                return cen_[x * 3 + axis] < cen_[y * 3 + axis];
            });
        }

        const int l = node_count_.fetch_add(2);
        nd.left = l;
        nd.right = l + 1;
        nd.count = 0;
        const uint32_t lcount = mid - b;
        if(count > 200000 && live_threads_.load() < threads_)
        {
            live_threads_.fetch_add(1);
            std::thread th([this, l, b, mid, depth] { build(l, b, mid, depth + 1); });
            build(l + 1, mid, e, depth + 1);
            th.join();
            live_threads_.fetch_sub(1);
        }
        else
        {
            (void)lcount;
            build(l, b, mid, depth + 1);
            build(l + 1, mid, e, depth + 1);
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

} // namespace

CWBVH build_cwbvh(const std::vector<TriRec> &tris, int threads)
{
    CWBVH out;
    if(tris.empty())
        return out;
    if(threads <= 0)
        threads = std::max(1u, std::thread::hardware_concurrency());

    BinaryBuilder bb(tris, threads);
    bb.run();
    const std::vector<BNode> &bn = bb.nodes_;
    out.binary_nodes = static_cast<int>(bn.size());

    // Wide collapse by dynamic programming over the binary tree (Ylitie, Karras and
    // Laine, "Efficient incoherent ray traversal on GPUs through compressed wide BVHs",
    // HPG 2017, section 3): C(n, i) is the least SAH cost of the subtree of n spread over
    // at most i child slots of a wide node; one slot holds either a leaf of <= 3
    // triangles or a wide node whose 8 slots hold the subtree. Children have larger
    // indices than their parents, so one reverse sweep visits the tree bottom-up.
    const size_t N = bn.size();
    std::vector<uint32_t> ntri(N);
    std::vector<float> cost(N * 8);
    std::vector<uint8_t> split(N * 8, 0);    // [n][i-1], i >= 2: left share k, 0: same as i - 1
    std::vector<uint8_t> split8(N, 0);       // left share of the 8-slot distribution
    std::vector<uint8_t> as_leaf(N, 0);
    const float INF = std::numeric_limits<float>::infinity();
    for(size_t q = N; q-- > 0;)
    {
        const BNode &nd = bn[q];
        const float A = static_cast<float>(nd.box.area());
        float *c = &cost[q * 8];
        if(nd.left < 0)
        {
            ntri[q] = nd.count;
            as_leaf[q] = 1;
            for(int i = 0; i < 8; ++i)
                c[i] = A * WIDE_COST_TRI * static_cast<float>(nd.count);
            continue;
        }
        ntri[q] = ntri[nd.left] + ntri[nd.right];
        const float *cl = &cost[static_cast<size_t>(nd.left) * 8], *cr = &cost[static_cast<size_t>(nd.right) * 8];
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
        split8[q] = arg[8];
        const float c_internal = A * WIDE_COST_NODE + dist[8];
        const float c_leaf = ntri[q] <= MAX_LEAF ? A * WIDE_COST_TRI * static_cast<float>(ntri[q]) : INF;
        as_leaf[q] = c_leaf <= c_internal ? 1 : 0;
        c[0] = std::min(c_leaf, c_internal);
        for(int i = 2; i <= 8; ++i)
        {
            if(dist[i] < c[i - 2])
            {
                c[i - 1] = dist[i];
                split[q * 8 + i - 1] = arg[i];
            }
            else
                c[i - 1] = c[i - 2];
        }
    }
    // the slots a subtree takes when it may use up to i of them
    auto expand = [&](auto &&self, int m, int i, std::vector<int> &out) -> void {
        while(i >= 2 && split[static_cast<size_t>(m) * 8 + i - 1] == 0)
            --i;
        if(i == 1)
        {
            out.push_back(m);
            return;
        }
        const int k = split[static_cast<size_t>(m) * 8 + i - 1];
        self(self, bn[m].left, k, out);
        self(self, bn[m].right, i - k, out);
    };
    // triangles (binary-leaf ranges) of a subtree kept as one leaf slot
    auto leaf_tris = [&](int m, std::vector<uint32_t> &out) {
        std::vector<int> st{ m };
        while(!st.empty())
        {
            const int x = st.back();
            st.pop_back();
            if(bn[x].left < 0)
            {
                for(uint32_t t = 0; t < bn[x].count; ++t)
                    out.push_back(bb.idx_[bn[x].first + t]);
            }
            else
            {
                st.push_back(bn[x].right);
                st.push_back(bn[x].left);
            }
        }
    };

    struct Job { int bnode; int wnode; int depth; };
    std::deque<Job> queue;
    out.nodes.reserve(bn.size() / 4 + 1);
    out.tris.reserve(tris.size());
    out.nodes.push_back(CWNode{});
    queue.push_back({ 0, 0, 1 });

    std::vector<int> kidv;
    std::vector<uint32_t> ltris;
    while(!queue.empty())
    {
        const Job job = queue.front();
        queue.pop_front();
        out.depth = std::max(out.depth, job.depth);

        // the wide node's children: the 8-slot distribution of the binary node's subtree
        kidv.clear();
        const BNode &root = bn[job.bnode];
        if(root.left < 0)
            kidv.push_back(job.bnode);
        else
        {
            const int k = split8[job.bnode];
            expand(expand, root.left, k, kidv);
            expand(expand, root.right, 8 - k, kidv);
        }
        int kids[8];
        const int nk = static_cast<int>(kidv.size());
        for(int k = 0; k < nk; ++k)
            kids[k] = kidv[k];

        // node origin and quantisation grid
        Box nbox;
        for(int k = 0; k < nk; ++k)
            nbox.grow(bn[kids[k]].box);
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

        // slot assignment: slot s prefers children far along (s&1?+x:-x, s&2?+y:-y, s&4?+z:-z);
        // the traversal visits slot == ray octant first
        double pc[3];
        for(int a = 0; a < 3; ++a)
            pc[a] = 0.5 * ((double)nbox.lo[a] + nbox.hi[a]);
        int slot_of[8];
        int kid_in_slot[8];
        for(int s = 0; s < 8; ++s)
            kid_in_slot[s] = -1;
        {
            double cost[8][8];
            for(int k = 0; k < nk; ++k)
            {
                const Box &cb = bn[kids[k]].box;
                double cc[3];
                for(int a = 0; a < 3; ++a)
                    cc[a] = 0.5 * ((double)cb.lo[a] + cb.hi[a]) - pc[a];
                for(int s = 0; s < 8; ++s)
                    cost[k][s] = ((s & 1) ? cc[0] : -cc[0]) + ((s & 2) ? cc[1] : -cc[1]) + ((s & 4) ? cc[2] : -cc[2]);
            }
            bool kid_done[8] = {};
            for(int round = 0; round < nk; ++round)
            {
                int bk = -1, bs = -1;
                double bc = -std::numeric_limits<double>::infinity();
                for(int k = 0; k < nk; ++k)
                {
                    if(kid_done[k])
                        continue;
                    for(int s = 0; s < 8; ++s)
                        if(kid_in_slot[s] < 0 && cost[k][s] > bc)
                        {
                            bc = cost[k][s];
                            bk = k;
                            bs = s;
                        }
                }
                kid_done[bk] = true;
                kid_in_slot[bs] = bk;
                slot_of[bk] = bs;
            }
        }

        // children in slot order: internal ones get consecutive wide nodes, leaf
        // triangles are appended contiguously
        int n_internal = 0;
        for(int s = 0; s < 8; ++s)
            if(kid_in_slot[s] >= 0 && !as_leaf[kids[kid_in_slot[s]]])
                ++n_internal;
        node.child_base = static_cast<uint32_t>(out.nodes.size());
        node.tri_base = static_cast<uint32_t>(out.tris.size());
        node.imask = 0;
        uint32_t tri_off = 0;
        int next_internal = 0;
        for(int s = 0; s < 8; ++s)
        {
            const int k = kid_in_slot[s];
            if(k < 0)
            {
                node.meta[s] = 0;
                continue;
            }
            const BNode &c = bn[kids[k]];
            // quantise (exact in double: power-of-two scale)
            const double lo[3] = { (double)c.box.lo[0], (double)c.box.lo[1], (double)c.box.lo[2] };
            const double hi[3] = { (double)c.box.hi[0], (double)c.box.hi[1], (double)c.box.hi[2] };
            const double org[3] = { (double)node.px, (double)node.py, (double)node.pz };
            uint8_t ql[3], qh[3];
            for(int a = 0; a < 3; ++a)
            {
                const double sc = std::ldexp(1.0, ex[a]);
                double l = std::floor((lo[a] - org[a]) / sc);
                double h = std::ceil((hi[a] - org[a]) / sc);
                l = std::max(0.0, std::min(255.0, l));
                h = std::max(0.0, std::min(255.0, h));
                ql[a] = static_cast<uint8_t>(l);
                qh[a] = static_cast<uint8_t>(h);
            }
            node.qlo_x[s] = ql[0]; node.qlo_y[s] = ql[1]; node.qlo_z[s] = ql[2];
            node.qhi_x[s] = qh[0]; node.qhi_y[s] = qh[1]; node.qhi_z[s] = qh[2];
            if(!as_leaf[kids[k]])
            {
                node.imask |= static_cast<uint8_t>(1u << s);
                node.meta[s] = static_cast<uint8_t>((1u << 5) | (24u + s));
                const int wn = static_cast<int>(node.child_base) + next_internal++;
                queue.push_back({ kids[k], wn, job.depth + 1 });
            }
            else
            {
                static const uint8_t unary[4] = { 0, 1, 3, 7 };
                ltris.clear();
                leaf_tris(kids[k], ltris);
                const uint32_t cnt = static_cast<uint32_t>(ltris.size());
                node.meta[s] = static_cast<uint8_t>((unary[cnt] << 5) | tri_off);
                for(uint32_t t : ltris)
                    out.tris.push_back(tris[t]);
                tri_off += cnt;
            }
        }
        (void)slot_of;
        for(int k = 0; k < n_internal; ++k)
            out.nodes.push_back(CWNode{});
        out.nodes[job.wnode] = node;
    }
    if(out.depth > TRAVERSAL_STACK_SIZE)
        throw std::runtime_error("BVH too deep for the traversal stack (" + std::to_string(out.depth) + " levels)");
    return out;
}

} // namespace bt
