// Binned-SAH BVH builder (host, multi-threaded top levels) and flattening to
// the device layout of bvh.h.
#include "bvh.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <future>
#include <limits>
#include <thread>

namespace dl {
namespace {

struct Box {
    float lo[3] = {std::numeric_limits<float>::infinity(), std::numeric_limits<float>::infinity(),
                   std::numeric_limits<float>::infinity()};
    float hi[3] = {-std::numeric_limits<float>::infinity(), -std::numeric_limits<float>::infinity(),
                   -std::numeric_limits<float>::infinity()};
    void grow(const float* p) {
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], p[k]);
            hi[k] = std::max(hi[k], p[k]);
        }
    }
    void grow(const Box& b) {
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    bool empty() const { return !(lo[0] <= hi[0]); }
    float area() const {
        if (empty()) return 0.f;
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return 2.f * (dx * dy + dy * dz + dz * dx);
    }
};

struct Prim {
    Box box;
    float c[3];
};

struct BuildNode {
    Box box;
    int left = -1, right = -1;   // children (build node indices); -1 for leaves
    int first = 0, count = 0;    // leaf range in `order`
    int depth = 0;
};

struct Builder {
    const BvhBuildOptions& opt;
    std::vector<Prim> prims;
    std::vector<int32_t> order;
    std::vector<BuildNode> nodes;
    std::atomic<int> next_node{0};
    std::atomic<int> max_depth{0};
    std::atomic<int> leaves{0};

    explicit Builder(const BvhBuildOptions& o) : opt(o) {}

    int alloc() { return next_node.fetch_add(1); }

    void make_leaf(int ni, int begin, int end, const Box& box, int depth) {
        BuildNode& nd = nodes[ni];
        nd.box = box;
        nd.first = begin;
        nd.count = end - begin;
        nd.depth = depth;
        leaves.fetch_add(1);
        int d = max_depth.load();
        while (depth > d && !max_depth.compare_exchange_weak(d, depth)) {
        }
    }

    // Builds node `ni` over order[begin, end).
    void build(int ni, int begin, int end, int depth) {
        Box box, cbox;
        for (int i = begin; i < end; i++) {
            const Prim& p = prims[order[i]];
            box.grow(p.box);
            cbox.grow(p.c);
        }
        int n = end - begin;
        if (n <= 1) {
            make_leaf(ni, begin, end, box, depth);
            return;
        }
        // binned SAH over the three axes
        const int B = opt.bins;
        float best_cost = std::numeric_limits<float>::infinity();
        int best_axis = -1, best_split = -1;
        float parent_area = box.area();
        std::vector<Box> bb(B);
        std::vector<int> cnt(B);
        std::vector<float> right_area(B);
        std::vector<int> right_cnt(B);
        for (int axis = 0; axis < 3; axis++) {
            float lo = cbox.lo[axis], hi = cbox.hi[axis];
            if (!(hi > lo)) continue;
            float scale = B / (hi - lo);
            std::fill(bb.begin(), bb.end(), Box());
            std::fill(cnt.begin(), cnt.end(), 0);
            for (int i = begin; i < end; i++) {
                const Prim& p = prims[order[i]];
                int b = std::min(B - 1, (int)((p.c[axis] - lo) * scale));
                bb[b].grow(p.box);
                cnt[b]++;
            }
            Box acc;
            int c = 0;
            for (int b = B - 1; b > 0; b--) {
                acc.grow(bb[b]);
                c += cnt[b];
                right_area[b] = acc.area();
                right_cnt[b] = c;
            }
            acc = Box();
            c = 0;
            for (int b = 0; b < B - 1; b++) {
                acc.grow(bb[b]);
                c += cnt[b];
                int rc = right_cnt[b + 1];
                if (c == 0 || rc == 0) continue;
                float cost = opt.traversal_cost +
                             opt.intersect_cost * (acc.area() * c + right_area[b + 1] * rc) /
                                 std::max(parent_area, 1e-30f);
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = axis;
                    best_split = b;
                }
            }
        }
        float leaf_cost = opt.intersect_cost * n;
        bool must_split = n > kMaxLeafTris;
        if (!must_split && (n <= opt.max_leaf_size && leaf_cost <= best_cost)) {
            make_leaf(ni, begin, end, box, depth);
            return;
        }
        if (!must_split && depth >= kMaxDepth) {
            make_leaf(ni, begin, end, box, depth);
            return;
        }
        int mid;
        if (best_axis >= 0 && depth < kMaxDepth) {
            float lo = cbox.lo[best_axis], hi = cbox.hi[best_axis];
            float scale = B / (hi - lo);
            auto it = std::partition(order.begin() + begin, order.begin() + end, [&](int32_t id) {
                int b = std::min(B - 1, (int)((prims[id].c[best_axis] - lo) * scale));
                return b <= best_split;
            });
            mid = (int)(it - order.begin());
            if (mid == begin || mid == end) mid = begin + n / 2;
        } else {
            // no usable SAH split (coincident centroids or depth cap): object median
            int axis = 0;
            float ext = -1;
            for (int k = 0; k < 3; k++)
                if (cbox.hi[k] - cbox.lo[k] > ext) {
                    ext = cbox.hi[k] - cbox.lo[k];
                    axis = k;
                }
            mid = begin + n / 2;
            std::nth_element(order.begin() + begin, order.begin() + mid, order.begin() + end,
                             [&](int32_t a, int32_t b) { return prims[a].c[axis] < prims[b].c[axis]; });
        }
        int l = alloc(), r = alloc();
        BuildNode& nd = nodes[ni];
        nd.box = box;
        nd.left = l;
        nd.right = r;
        nd.count = 0;
        nd.depth = depth;
        if (n > 65536) {
            auto fut = std::async(std::launch::async, [&, l, begin, mid, depth] { build(l, begin, mid, depth + 1); });
            build(r, mid, end, depth + 1);
            fut.get();
        } else {
            build(l, begin, mid, depth + 1);
            build(r, mid, end, depth + 1);
        }
    }
};

// Grow a box outwards by a few ulps of its magnitude so the float slab test
// on the device never rejects a triangle that the exact test hits.
void pad(float& lo, float& hi) {
    float m = std::max(std::fabs(lo), std::fabs(hi));
    float e = m * 2.4e-7f + 1e-30f;
    lo -= e;
    hi += e;
}

}  // namespace

BvhResult build_bvh(const float* tris, int64_t n, const BvhBuildOptions& opt) {
    auto t0 = std::chrono::steady_clock::now();
    BvhResult res;
    Builder b(opt);
    b.prims.resize(n);
    b.order.resize(n);
    for (int64_t i = 0; i < n; i++) {
        Prim& p = b.prims[i];
        const float* v = tris + 9 * i;
        p.box.grow(v);
        p.box.grow(v + 3);
        p.box.grow(v + 6);
        for (int k = 0; k < 3; k++) p.c[k] = 0.5f * (p.box.lo[k] + p.box.hi[k]);
        b.order[i] = (int32_t)i;
    }
    b.nodes.resize(std::max<int64_t>(2 * n + 1, 1));
    int root = b.alloc();
    if (n > 0) b.build(root, 0, (int)n, 0);
    int nb = b.next_node.load();

    // Flatten: inner nodes in depth-first order, triangles in leaf order.
    std::vector<int> gpu_index(nb, -1);
    std::vector<int> stack;
    // Root: if the whole tree is one leaf (or empty), wrap it in an inner node.
    const BuildNode& R = b.nodes[root];
    auto leaf_ref = [&](const BuildNode& nd) -> int32_t {
        int first = (int)res.tris.size();
        for (int i = 0; i < nd.count; i++) {
            int32_t id = b.order[nd.first + i];
            GpuTri t;
            std::memcpy(t.v0, tris + 9 * id, 12);
            std::memcpy(t.v1, tris + 9 * id + 3, 12);
            std::memcpy(t.v2, tris + 9 * id + 6, 12);
            t.prim = id;
            t.mat_type = t.pad2 = 0;
            res.tris.push_back(t);
            res.tri_order.push_back(id);
        }
        return ~((first << 4) | (nd.count - 1));
    };
    auto set_child = [&](GpuNode& g, int slot, const Box& bx, int32_t ref) {
        float lo[3], hi[3];
        for (int k = 0; k < 3; k++) {
            lo[k] = bx.lo[k];
            hi[k] = bx.hi[k];
            if (!bx.empty()) pad(lo[k], hi[k]);
        }
        if (slot == 0) {
            g.a[0] = lo[0]; g.a[1] = hi[0]; g.a[2] = lo[1]; g.a[3] = hi[1];
            g.c[0] = lo[2]; g.c[1] = hi[2];
        } else {
            g.b[0] = lo[0]; g.b[1] = hi[0]; g.b[2] = lo[1]; g.b[3] = hi[1];
            g.c[2] = lo[2]; g.c[3] = hi[2];
        }
        g.d[slot] = ref;
    };
    GpuNode empty_node;
    std::memset(&empty_node, 0, sizeof(empty_node));
    Box nobox;
    if (n == 0 || R.left < 0) {
        // a one-leaf tree references its leaf from both slots (the traversal
        // kernels take both children of a node as present); an empty tree's
        // root is never visited
        GpuNode g = empty_node;
        const int32_t ref = n > 0 ? leaf_ref(R) : kEmptyRef;
        set_child(g, 0, n > 0 ? R.box : nobox, ref);
        set_child(g, 1, n > 0 ? R.box : nobox, ref);
        res.nodes.push_back(g);
        res.depth = 1;
        res.leaves = n > 0 ? 1 : 0;
    } else {
        // iterative DFS: node emitted, then its left subtree, then its right
        struct Item { int bn; int parent; int slot; };
        std::vector<Item> st;
        st.push_back({root, -1, 0});
        while (!st.empty()) {
            Item it = st.back();
            st.pop_back();
            const BuildNode& nd = b.nodes[it.bn];
            int32_t ref;
            if (nd.left < 0) {
                ref = leaf_ref(nd);
            } else {
                ref = (int32_t)res.nodes.size();
                res.nodes.push_back(empty_node);
                st.push_back({nd.right, ref, 1});
                st.push_back({nd.left, ref, 0});
            }
            if (it.parent >= 0) set_child(res.nodes[it.parent], it.slot, nd.box, ref);
        }
        res.depth = b.max_depth.load() + 1;
        res.leaves = b.leaves.load();
    }
    // SAH cost of the result (relative to the root box)
    if (n > 0) {
        double ra = std::max(R.box.area(), 1e-30f);
        double cost = 0;
        for (int i = 0; i < nb; i++) {
            const BuildNode& nd = b.nodes[i];
            if (nd.left >= 0)
                cost += opt.traversal_cost * nd.box.area() / ra;
            else
                cost += opt.intersect_cost * nd.count * nd.box.area() / ra;
        }
        res.sah_cost = cost;
    }
    res.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return res;
}

}  // namespace dl
