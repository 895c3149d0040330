// rt_bvh.cpp -- binned-SAH build of the device BVH2 (see rt_bvh.h).
//
// The reference builds a binary SAH BVH per mesh and a second one over the
// meshes (accelStruct/Bvh.cpp:51-79, :611-771; factory/MeshFactory.h:123,
// core/Scene.cpp:117).  The device tracer flattens every mesh into one tree:
// closest-hit results are independent of the tree shape (only exactly equal
// hit distances on different triangles depend on visit order), and a single
// tree avoids traversing overlapping per-mesh trees.
#include "rt_bvh.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <future>

namespace rtgpu {

namespace {

struct Box {
    float mn[3], mx[3];
    void reset() { for (int i = 0; i < 3; i++) { mn[i] = INFINITY; mx[i] = -INFINITY; } }
    void grow(const Box &b) { for (int i = 0; i < 3; i++) { mn[i] = std::min(mn[i], b.mn[i]); mx[i] = std::max(mx[i], b.mx[i]); } }
    void grow(const float *p) { for (int i = 0; i < 3; i++) { mn[i] = std::min(mn[i], p[i]); mx[i] = std::max(mx[i], p[i]); } }
    double area() const
    {
        double dx = (double)mx[0] - mn[0], dy = (double)mx[1] - mn[1], dz = (double)mx[2] - mn[2];
        if (dx < 0 || dy < 0 || dz < 0) return 0.0;
        return 2.0 * (dx * dy + dy * dz + dz * dx);
    }
};

struct BuildNode {
    Box box;
    int child[2] = {-1, -1};   // indices into the build-node array
    int first = 0, count = 0;  // leaf range into the order array
    bool leaf = false;
};

struct Builder {
    const float *tv;
    std::vector<Box> tb;
    std::vector<float> cen;   // 3 per triangle
    std::vector<int> order;
    int max_leaf, n_bins;

    // Build subtree over order[b, e); returns nodes appended into `out`
    // (local indices) with the subtree root first.
    void build(int b, int e, std::vector<BuildNode> &out, int depth, int &maxd)
    {
        maxd = std::max(maxd, depth);
        int self = (int)out.size();
        out.emplace_back();
        Box box, cb;
        box.reset(); cb.reset();
        for (int i = b; i < e; i++) {
            box.grow(tb[order[i]]);
            cb.grow(&cen[3 * (size_t)order[i]]);
        }
        out[self].box = box;
        int n = e - b;
        if (n <= 1) { out[self].leaf = true; out[self].first = b; out[self].count = n; return; }
        // binned SAH over the centroid bounds
        int best_axis = -1, best_bin = -1;
        double best_cost = INFINITY;
        const int NB = n_bins;
        std::vector<Box> bb(NB);
        std::vector<int> bc(NB);
        std::vector<double> la(NB), ra(NB);
        std::vector<int> lc(NB), rc(NB);
        for (int a = 0; a < 3; a++) {
            float lo = cb.mn[a], hi = cb.mx[a];
            if (!(hi > lo)) continue;
            double sc = NB / ((double)hi - lo);
            for (int k = 0; k < NB; k++) { bb[k].reset(); bc[k] = 0; }
            for (int i = b; i < e; i++) {
                int t = order[i];
                int k = std::min(NB - 1, (int)(((double)cen[3 * (size_t)t + a] - lo) * sc));
                bb[k].grow(tb[t]);
                bc[k]++;
            }
            Box acc; acc.reset(); int cnt = 0;
            for (int k = 0; k < NB - 1; k++) { acc.grow(bb[k]); cnt += bc[k]; la[k] = acc.area(); lc[k] = cnt; }
            acc.reset(); cnt = 0;
            for (int k = NB - 1; k > 0; k--) { acc.grow(bb[k]); cnt += bc[k]; ra[k - 1] = acc.area(); rc[k - 1] = cnt; }
            for (int k = 0; k < NB - 1; k++) {
                if (lc[k] == 0 || rc[k] == 0) continue;
                double c = la[k] * lc[k] + ra[k] * rc[k];
                if (c < best_cost) { best_cost = c; best_axis = a; best_bin = k; }
            }
        }
        double parea = box.area();
        double leaf_cost = (double)n;
        double split_cost = parea > 0 ? 1.0 + best_cost / parea : INFINITY;
        if (n <= max_leaf && (best_axis < 0 || leaf_cost <= split_cost)) {
            out[self].leaf = true; out[self].first = b; out[self].count = n;
            return;
        }
        int mid;
        if (best_axis < 0) {
            // all centroids coincide: split the range in the middle
            mid = b + n / 2;
        } else {
            float lo = cb.mn[best_axis], hi = cb.mx[best_axis];
            double sc = NB / ((double)hi - lo);
            int a = best_axis;
            int *pm = std::partition(order.data() + b, order.data() + e, [&](int t) {
                int k = std::min(NB - 1, (int)(((double)cen[3 * (size_t)t + a] - lo) * sc));
                return k <= best_bin;
            });
            mid = (int)(pm - order.data());
            if (mid == b || mid == e) mid = b + n / 2;
        }
        // large subtrees build their children in parallel
        if (n > 200000) {
            std::vector<BuildNode> left, right;
            int md1 = 0, md2 = 0;
            auto fut = std::async(std::launch::async, [&]() { build(b, mid, left, depth + 1, md1); });
            build(mid, e, right, depth + 1, md2);
            fut.get();
            maxd = std::max(maxd, std::max(md1, md2));
            int lbase = (int)out.size();
            for (auto &nd : left) {
                if (!nd.leaf) { nd.child[0] += lbase; nd.child[1] += lbase; }
                out.push_back(nd);
            }
            int rbase = (int)out.size();
            for (auto &nd : right) {
                if (!nd.leaf) { nd.child[0] += rbase; nd.child[1] += rbase; }
                out.push_back(nd);
            }
            out[self].child[0] = lbase;
            out[self].child[1] = rbase;
        } else {
            int l = (int)out.size();
            build(b, mid, out, depth + 1, maxd);
            int r = (int)out.size();
            build(mid, e, out, depth + 1, maxd);
            out[self].child[0] = l;
            out[self].child[1] = r;
        }
    }
};

// widen a box outward so the fused slab test stays conservative
inline void widen(const Box &b, float scale_eps, float out[6])
{
    for (int i = 0; i < 3; i++) {
        float ext = b.mx[i] - b.mn[i];
        float m = std::max(std::fabs(b.mn[i]), std::fabs(b.mx[i]));
        float pad = ext * 1e-6f + m * 1.2e-6f + scale_eps;
        out[2 * i] = b.mn[i] - pad;
        out[2 * i + 1] = b.mx[i] + pad;
    }
}

}  // namespace

void build_bvh2(const float *tv, int n, BvhImage &img, int max_leaf, int n_bins)
{
    img = BvhImage();
    if (n <= 0) return;
    max_leaf = std::max(1, std::min(max_leaf, 8));
    Builder B;
    B.tv = tv;
    B.max_leaf = max_leaf;
    B.n_bins = n_bins;
    B.tb.resize(n);
    B.cen.resize(3 * (size_t)n);
    B.order.resize(n);
    Box scene; scene.reset();
    for (int t = 0; t < n; t++) {
        Box b; b.reset();
        for (int k = 0; k < 3; k++) b.grow(tv + 9 * (size_t)t + 3 * k);
        B.tb[t] = b;
        scene.grow(b);
        for (int a = 0; a < 3; a++) B.cen[3 * (size_t)t + a] = 0.5f * (b.mn[a] + b.mx[a]);
        B.order[t] = t;
    }
    float sext = 0.f;
    for (int a = 0; a < 3; a++) sext = std::max(sext, scene.mx[a] - scene.mn[a]);
    float seps = std::max(sext * 1e-7f, 1e-30f);
    std::vector<BuildNode> bn;
    bn.reserve(2 * (size_t)n / std::max(1, max_leaf) + 16);
    int maxd = 0;
    B.build(0, n, bn, 0, maxd);
    // leaves larger than 8 cannot be encoded: split them (only happens for
    // n > max_leaf with identical centroids, handled by the mid split above)
    // Map build nodes -> device internal nodes.  A root leaf gets a
    // synthetic internal parent with an empty second child.
    std::vector<int> dev_index(bn.size(), -1);
    int n_int = 0;
    for (size_t i = 0; i < bn.size(); i++) if (!bn[i].leaf) dev_index[i] = n_int++;
    bool root_leaf = bn[0].leaf;
    if (root_leaf) n_int = 1;
    img.n_nodes = n_int;
    img.nodes.assign(16 * (size_t)n_int, 0.f);
    img.n_slots = n;
    img.tri_slots.assign(12 * (size_t)n, 0.f);
    for (int s = 0; s < n; s++) {
        int t = B.order[s];
        const float *p = tv + 9 * (size_t)t;
        float *o = &img.tri_slots[12 * (size_t)s];
        int32_t id = t;
        o[0] = p[0]; o[1] = p[1]; o[2] = p[2]; std::memcpy(&o[3], &id, 4);
        o[4] = p[3] - p[0]; o[5] = p[4] - p[1]; o[6] = p[5] - p[2]; o[7] = 0.f;
        o[8] = p[6] - p[0]; o[9] = p[7] - p[1]; o[10] = p[8] - p[2]; o[11] = 0.f;
    }
    auto link = [&](int bi) -> int32_t {
        const BuildNode &c = bn[bi];
        if (!c.leaf) return dev_index[bi];
        int32_t enc = (c.first << 3) | (std::max(1, c.count) - 1);
        return ~enc;
    };
    auto write_node = [&](int di, const Box &b0, int32_t l0, const Box &b1, int32_t l1, bool empty1) {
        float w0[6], w1[6];
        widen(b0, seps, w0);
        if (empty1) { for (int i = 0; i < 3; i++) { w1[2 * i] = INFINITY; w1[2 * i + 1] = -INFINITY; } }
        else widen(b1, seps, w1);
        float *o = &img.nodes[16 * (size_t)di];
        o[0] = w0[0]; o[1] = w0[1]; o[2] = w0[2]; o[3] = w0[3];
        o[4] = w1[0]; o[5] = w1[1]; o[6] = w1[2]; o[7] = w1[3];
        o[8] = w0[4]; o[9] = w0[5]; o[10] = w1[4]; o[11] = w1[5];
        std::memcpy(&o[12], &l0, 4);
        std::memcpy(&o[13], &l1, 4);
        o[14] = 0.f; o[15] = 0.f;
    };
    double sah = 0.0;
    double ra = bn[0].box.area();
    if (root_leaf) {
        write_node(0, bn[0].box, link(0), bn[0].box, link(0), true);
    } else {
        for (size_t i = 0; i < bn.size(); i++) {
            const BuildNode &nd = bn[i];
            if (nd.leaf) { if (ra > 0) sah += nd.box.area() / ra * nd.count; continue; }
            if (ra > 0) sah += nd.box.area() / ra;
            write_node(dev_index[i], bn[nd.child[0]].box, link(nd.child[0]), bn[nd.child[1]].box, link(nd.child[1]), false);
        }
    }
    img.max_depth = maxd;
    img.sah_cost = sah;
}

}  // namespace rtgpu
