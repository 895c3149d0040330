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
#include <array>
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
    double c_node = 1.0;   // SAH cost of a node visit, in triangle tests
    int depth_cap = RT_BVH_DEPTH_CAP;

    static int ceil_log2(int n)
    {
        int k = 0;
        while ((int64_t(1) << k) < n) k++;
        return k;
    }

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
        int mid;
        // Depth bound.  Once depth + ceil(log2 n) reaches the cap, the subtree
        // is split at the object median along the widest centroid axis: each
        // child then holds at most ceil(n/2) triangles, so every leaf ends at
        // depth <= depth_cap and the traversal stacks (one entry per level)
        // cannot overflow.  The parent of the first capped node was below the
        // cap with more triangles, so depth + ceil(log2 n) <= depth_cap there.
        // SAH trees of ordinary scenes never reach it; a scene whose SAH would
        // peel one triangle per level (sizes growing geometrically) does.
        if (depth + ceil_log2(n) >= depth_cap) {
            if (n <= max_leaf) { out[self].leaf = true; out[self].first = b; out[self].count = n; return; }
            int a = 0;
            for (int k = 1; k < 3; k++)
                if (cb.mx[k] - cb.mn[k] > cb.mx[a] - cb.mn[a]) a = k;
            mid = b + n / 2;
            std::nth_element(order.data() + b, order.data() + mid, order.data() + e, [&](int x, int y) {
                float cx = cen[3 * (size_t)x + a], cy = cen[3 * (size_t)y + a];
                return cx < cy || (cx == cy && x < y);
            });
            int l = (int)out.size();
            build(b, mid, out, depth + 1, maxd);
            int r = (int)out.size();
            build(mid, e, out, depth + 1, maxd);
            out[self].child[0] = l;
            out[self].child[1] = r;
            return;
        }
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
        double split_cost = parea > 0 ? c_node + best_cost / parea : INFINITY;
        if (n <= max_leaf && (best_axis < 0 || leaf_cost <= split_cost)) {
            out[self].leaf = true; out[self].first = b; out[self].count = n;
            return;
        }
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

// The device image of a built tree: internal nodes in build order (a root
// leaf gets a synthetic parent with an empty second child), triangle slots
// in leaf order, boxes widened.
static void write_image(const float *tv, int n, const std::vector<BuildNode> &bn, const std::vector<int> &order,
                        float seps, int maxd, BvhImage &img)
{
    // Leaves hold at most 8 triangles (a link encodes count - 1 in 3 bits);
    // both builders guarantee it.  Build nodes map to device internal nodes;
    // a root leaf gets a synthetic internal parent with an empty second child.
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
        int t = order[s];
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

void build_bvh2(const float *tv, int n, BvhImage &img, int max_leaf, int n_bins, double c_node, int depth_cap)
{
    img = BvhImage();
    if (n <= 0) return;
    max_leaf = std::max(1, std::min(max_leaf, 8));
    Builder B;
    B.depth_cap = depth_cap;
    B.tv = tv;
    B.max_leaf = max_leaf;
    B.n_bins = n_bins;
    B.c_node = c_node;
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
    write_image(tv, n, bn, B.order, seps, maxd, img);
}

namespace {

struct Collapse {
    const std::vector<BuildNode> &bn;
    const std::vector<int> &order;
    const float *tv;
    float seps;
    WideBvhImage &img;
    int maxd = 0;

    Collapse(const std::vector<BuildNode> &b, const std::vector<int> &o, const float *t, float e, WideBvhImage &im)
        : bn(b), order(o), tv(t), seps(e), img(im) {}

    void push_tri(int t)
    {
        const float *p = tv + 9 * (size_t)t;
        float o[12];
        int32_t id = t;
        o[0] = p[0]; o[1] = p[1]; o[2] = p[2]; std::memcpy(&o[3], &id, 4);
        o[4] = p[3] - p[0]; o[5] = p[4] - p[1]; o[6] = p[5] - p[2]; o[7] = 0.f;
        o[8] = p[6] - p[0]; o[9] = p[7] - p[1]; o[10] = p[8] - p[2]; o[11] = 0.f;
        img.tri_slots.insert(img.tri_slots.end(), o, o + 12);
        img.n_slots++;
    }

    // quantise [lo, hi] outward on a grid p + q * s, q in [0, 255]
    static void quant(float p, float s, float lo, float hi, uint8_t &qlo, uint8_t &qhi)
    {
        int a = (int)std::floor(((double)lo - p) / s);
        int b = (int)std::ceil(((double)hi - p) / s);
        a = std::max(0, std::min(255, a));
        b = std::max(0, std::min(255, b));
        // decoded with binary32 arithmetic the box must still contain [lo, hi]
        while (a > 0 && p + (float)a * s > lo) a--;
        while (b < 255 && p + (float)b * s < hi) b++;
        qlo = (uint8_t)a;
        qhi = (uint8_t)b;
    }

    void emit(int wi, int bi, int depth)
    {
        maxd = std::max(maxd, depth);
        std::vector<int> ch;
        if (bn[bi].leaf) ch.push_back(bi);
        else { ch.push_back(bn[bi].child[0]); ch.push_back(bn[bi].child[1]); }
        while ((int)ch.size() < 8) {
            int best = -1;
            double ba = -1.0;
            for (int k = 0; k < (int)ch.size(); k++) {
                const BuildNode &c = bn[ch[k]];
                if (c.leaf) continue;
                double a = c.box.area();
                if (a > ba) { ba = a; best = k; }
            }
            if (best < 0) break;
            int b = ch[best];
            ch[best] = bn[b].child[0];
            ch.insert(ch.begin() + best + 1, bn[b].child[1]);
        }
        // widened child boxes and the node box
        float cb[8][6];
        Box nb; nb.reset();
        for (int k = 0; k < (int)ch.size(); k++) {
            widen(bn[ch[k]].box, seps, cb[k]);
            Box w;
            for (int a = 0; a < 3; a++) { w.mn[a] = cb[k][2 * a]; w.mx[a] = cb[k][2 * a + 1]; }
            nb.grow(w);
        }
        // The device evaluates a plane as fma(q, 2^e * idir, p * idir - o * idir):
        // besides the origin term (covered by the traversal's slab guard) it rounds
        // values up to |p| + extent of this node, so pad every child by that.
        for (int a = 0; a < 3; a++) {
            float npad = 2.5e-7f * (2.f * std::fabs(nb.mn[a]) + std::fabs(nb.mx[a]) + (nb.mx[a] - nb.mn[a]));
            for (int k = 0; k < (int)ch.size(); k++) { cb[k][2 * a] -= npad; cb[k][2 * a + 1] += npad; }
            nb.mn[a] -= npad; nb.mx[a] += npad;
        }
        float p[3], sc[3];
        uint8_t e[3];
        for (int a = 0; a < 3; a++) {
            p[a] = nb.mn[a];
            double ext = (double)nb.mx[a] - nb.mn[a];
            int ex = -126;
            if (ext > 0) {
                ex = (int)std::ceil(std::log2(ext / 255.0 * (1.0 + 1e-6)));
                while (std::ldexp(255.0, ex) < ext) ex++;
            }
            ex = std::max(-126, std::min(127, ex));
            // the top quantum must reach the node's max in binary32 too
            while (ex < 127 && p[a] + (float)std::ldexp(255.0, ex) < nb.mx[a]) ex++;
            sc[a] = (float)std::ldexp(1.0, ex);
            e[a] = (uint8_t)(ex + 127);
        }
        // Octant slots: slot s holds the child met first by rays whose
        // direction has sign bits s (bit a set: negative along axis a), i.e.
        // the child with the smallest centroid offset along that direction.
        // Rays visit slots in the order k ^ octant, k = 0..7.
        const int nc = (int)ch.size();
        int slot_of[8];
        {
            double cost[8][8];
            for (int k = 0; k < nc; k++) {
                double c[3];
                for (int a = 0; a < 3; a++)
                    c[a] = 0.5 * ((double)cb[k][2 * a] + cb[k][2 * a + 1]) - 0.5 * ((double)nb.mn[a] + nb.mx[a]);
                for (int sl = 0; sl < 8; sl++)
                    cost[k][sl] = (sl & 1 ? -c[0] : c[0]) + (sl & 2 ? -c[1] : c[1]) + (sl & 4 ? -c[2] : c[2]);
            }
            bool kused[8] = {false}, sused[8] = {false};
            for (int it = 0; it < nc; it++) {
                int bk = -1, bs = -1;
                double bc = 0.0;
                for (int k = 0; k < nc; k++) {
                    if (kused[k]) continue;
                    for (int sl = 0; sl < 8; sl++)
                        if (!sused[sl] && (bk < 0 || cost[k][sl] < bc)) { bk = k; bs = sl; bc = cost[k][sl]; }
                }
                kused[bk] = true; sused[bs] = true;
                slot_of[bk] = bs;
            }
        }
        int n_int = 0;
        for (int c : ch) if (!bn[c].leaf) n_int++;
        int child_base = img.n_nodes;
        img.n_nodes += n_int;
        img.nodes.resize(20 * (size_t)img.n_nodes, 0.f);
        int tri_base = img.n_slots;
        // empty slots: inverted boxes (lo 255 > hi 0) that no ray enters
        uint8_t meta[8] = {0, 0, 0, 0, 0, 0, 0, 0}, ql[3][8], qh[3][8];
        std::memset(ql, 255, sizeof(ql));
        std::memset(qh, 0, sizeof(qh));
        std::vector<std::pair<int, int>> inner;   // (wide index, binary index)
        int ki = 0;
        for (int sl = 0; sl < 8; sl++) {
            int k = -1;
            for (int j = 0; j < nc; j++) if (slot_of[j] == sl) k = j;
            if (k < 0) continue;
            const BuildNode &c = bn[ch[k]];
            for (int a = 0; a < 3; a++) quant(p[a], sc[a], cb[k][2 * a], cb[k][2 * a + 1], ql[a][sl], qh[a][sl]);
            if (c.leaf) {
                int off = img.n_slots - tri_base;
                for (int t = 0; t < c.count; t++) push_tri(order[c.first + t]);
                meta[sl] = (uint8_t)((std::max(1, c.count) << 5) | off);
            } else {
                meta[sl] = (uint8_t)(0xE0 | ki);
                inner.push_back({child_base + ki, ch[k]});
                ki++;
            }
        }
        float *o = &img.nodes[20 * (size_t)wi];
        uint32_t ebits = (uint32_t)e[0] | ((uint32_t)e[1] << 8) | ((uint32_t)e[2] << 16);
        o[0] = p[0]; o[1] = p[1]; o[2] = p[2]; std::memcpy(&o[3], &ebits, 4);
        int32_t cbv = child_base, tbv = tri_base;
        std::memcpy(&o[4], &cbv, 4);
        std::memcpy(&o[5], &tbv, 4);
        std::memcpy(&o[6], meta, 4);
        std::memcpy(&o[7], meta + 4, 4);
        std::memcpy(&o[8], ql[0], 8);
        std::memcpy(&o[10], ql[1], 8);
        std::memcpy(&o[12], ql[2], 8);
        std::memcpy(&o[14], qh[0], 8);
        std::memcpy(&o[16], qh[1], 8);
        std::memcpy(&o[18], qh[2], 8);
        for (auto &pr : inner) emit(pr.first, pr.second, depth + 1);
    }
};

}  // namespace

void build_wbvh8(const float *tv, int n, WideBvhImage &img, int n_bins, int depth_cap)
{
    img = WideBvhImage();
    if (n <= 0) return;
    Builder B;
    B.tv = tv;
    B.max_leaf = 3;
    B.n_bins = n_bins;
    B.depth_cap = depth_cap;
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
    bn.reserve(2 * (size_t)n / 2 + 16);
    int maxd = 0;
    B.build(0, n, bn, 0, maxd);
    img.tri_slots.reserve(12 * (size_t)n);
    img.n_nodes = 1;
    img.nodes.assign(20, 0.f);
    Collapse cl(bn, B.order, tv, seps, img);
    cl.emit(0, 0, 0);
    img.max_depth = cl.maxd;
}

void build_bvh4(const BvhImage &b2, Bvh4Image &out)
{
    out = Bvh4Image();
    if (b2.n_nodes <= 0) return;
    // one child entry of a binary node: its box (the six widened planes as
    // stored) and its link
    struct Entry { float pl[6]; int32_t link; double area; int32_t src; };
    auto entry = [&](int node, int k, Entry &e) -> bool {
        const float *o = &b2.nodes[16 * (size_t)node];
        if (k == 0) { e.pl[0] = o[0]; e.pl[1] = o[1]; e.pl[2] = o[2]; e.pl[3] = o[3]; e.pl[4] = o[8]; e.pl[5] = o[9]; }
        else { e.pl[0] = o[4]; e.pl[1] = o[5]; e.pl[2] = o[6]; e.pl[3] = o[7]; e.pl[4] = o[10]; e.pl[5] = o[11]; }
        std::memcpy(&e.link, &o[12 + k], 4);
        e.src = 2 * node + k;
        // the empty second child of a root leaf: an inverted box
        if (!(e.pl[0] <= e.pl[1])) return false;
        double dx = (double)e.pl[1] - e.pl[0], dy = (double)e.pl[3] - e.pl[2], dz = (double)e.pl[5] - e.pl[4];
        e.area = 2.0 * (dx * dy + dy * dz + dz * dx);
        return true;
    };
    // breadth-first: a queue of (binary node, 4-wide node index, depth)
    struct Work { int node, wi, depth; };
    std::vector<Work> q;
    q.push_back({0, 0, 0});
    out.n_nodes = 1;
    out.nodes.assign(32, INFINITY);
    out.src.assign(4, -1);
    for (size_t h = 0; h < q.size(); h++) {
        const Work w = q[h];
        out.max_depth = std::max(out.max_depth, w.depth);
        Entry ch[4];
        int nc = 0;
        for (int k = 0; k < 2; k++)
            if (entry(w.node, k, ch[nc])) nc++;
        while (nc < 4) {
            int best = -1;
            for (int i = 0; i < nc; i++)
                if (ch[i].link >= 0 && (best < 0 || ch[i].area > ch[best].area)) best = i;
            if (best < 0) break;
            const int nb = ch[best].link;
            Entry a, b;
            bool ha = entry(nb, 0, a), hb = entry(nb, 1, b);
            if (ha && hb) { ch[best] = a; ch[nc++] = b; }
            else if (ha) ch[best] = a;
            else if (hb) ch[best] = b;
            else { ch[best] = ch[--nc]; }
        }
        float *o = &out.nodes[32 * (size_t)w.wi];
        for (int i = 0; i < 4; i++) {
            int32_t link = 0x7fffffff;
            if (i < nc) {
                for (int pl = 0; pl < 6; pl++) o[4 * pl + i] = ch[i].pl[pl];
                out.src[4 * (size_t)w.wi + i] = ch[i].src;
                link = ch[i].link;
                if (link >= 0) {
                    const int wi = out.n_nodes++;
                    out.nodes.resize(32 * (size_t)out.n_nodes, INFINITY);
                    out.src.resize(4 * (size_t)out.n_nodes, -1);
                    o = &out.nodes[32 * (size_t)w.wi];   // the resize may move the array
                    q.push_back({link, wi, w.depth + 1});
                    link = wi;
                }
            }
            std::memcpy(&o[24 + i], &link, 4);
        }
        for (int i = 28; i < 32; i++) o[i] = 0.f;
    }
}

bool import_bvh2(const float *tv, int n, const ExtNode *nodes, int n_nodes, const int32_t *prims, int n_prims,
                 BvhImage &img, std::string *why, int depth_cap)
{
    img = BvhImage();
    auto bad = [&](const std::string &m) { if (why) *why = m; return false; };
    if (n <= 0) return n_nodes == 0 ? true : bad("a tree for a scene without triangles");
    if (n_nodes <= 0 || !nodes) return bad("no nodes");
    if (n_prims != n || !prims) return bad("the leaves must list every triangle once");
    // Walk the tree (explicit stack): every node once, leaves in depth-first
    // order, every triangle once.  A leaf of more than 8 triangles becomes a
    // balanced subtree over halves of its range.
    struct Item { int node; int first, count; int depth; int parent; int side; };
    std::vector<char> seen(n_nodes, 0), tri_seen(n, 0);
    std::vector<BuildNode> bn;          // the tree as build_bvh2 would produce it
    std::vector<int> order;             // triangle per slot
    order.reserve(n);
    std::vector<Item> todo;
    todo.push_back({0, 0, 0, 0, -1, 0});
    int maxd = 0;
    while (!todo.empty()) {
        Item it = todo.back();
        todo.pop_back();
        int first = it.first, count = it.count;
        bool split_leaf = it.node < 0;   // a half of an oversized leaf
        if (!split_leaf) {
            if (it.node >= n_nodes) return bad("child index out of range");
            if (seen[it.node]) return bad("a node is reached twice");
            seen[it.node] = 1;
            const ExtNode &e = nodes[it.node];
            if (e.count < 0) return bad("negative leaf size");
            if (e.count == 0) {
                if (e.left < 0 || e.right < 0 || e.left >= n_nodes || e.right >= n_nodes)
                    return bad("internal node with a missing child");
                const int self = (int)bn.size();
                bn.emplace_back();
                if (it.parent >= 0) bn[it.parent].child[it.side] = self;
                maxd = std::max(maxd, it.depth);
                // right first on the stack, so the left subtree is laid out first
                todo.push_back({e.right, 0, 0, it.depth + 1, self, 1});
                todo.push_back({e.left, 0, 0, it.depth + 1, self, 0});
                continue;
            }
            if (e.first < 0 || (int64_t)e.first + e.count > n_prims) return bad("leaf range outside the triangle list");
            first = e.first;
            count = e.count;
        }
        if (count > 8) {
            const int self = (int)bn.size();
            bn.emplace_back();
            if (it.parent >= 0) bn[it.parent].child[it.side] = self;
            maxd = std::max(maxd, it.depth);
            const int h = count / 2;
            todo.push_back({-1, first + h, count - h, it.depth + 1, self, 1});
            todo.push_back({-1, first, h, it.depth + 1, self, 0});
            continue;
        }
        const int self = (int)bn.size();
        bn.emplace_back();
        if (it.parent >= 0) bn[it.parent].child[it.side] = self;
        maxd = std::max(maxd, it.depth);
        BuildNode &L = bn[self];
        L.leaf = true;
        L.first = (int)order.size();
        L.count = count;
        for (int k = 0; k < count; k++) {
            const int t = prims[first + k];
            if (t < 0 || t >= n) return bad("triangle index out of range");
            if (tri_seen[t]) return bad("a triangle is in two leaves");
            tri_seen[t] = 1;
            order.push_back(t);
        }
    }
    if ((int)order.size() != n) return bad("some triangles are in no leaf");
    if (maxd > depth_cap) return bad("deeper than the traversal stacks allow (" + std::to_string(maxd) + " levels)");
    // boxes bottom-up: children come after their parent in bn
    Box scene; scene.reset();
    for (int i = (int)bn.size() - 1; i >= 0; i--) {
        BuildNode &b = bn[i];
        b.box.reset();
        if (b.leaf) {
            for (int k = 0; k < b.count; k++)
                for (int c = 0; c < 3; c++) b.box.grow(tv + 9 * (size_t)order[b.first + k] + 3 * c);
        } else {
            b.box.grow(bn[b.child[0]].box);
            b.box.grow(bn[b.child[1]].box);
        }
    }
    scene = bn[0].box;
    float sext = 0.f;
    for (int a = 0; a < 3; a++) sext = std::max(sext, scene.mx[a] - scene.mn[a]);
    const float seps = std::max(sext * 1e-7f, 1e-30f);
    write_image(tv, n, bn, order, seps, maxd, img);
    return true;
}

bool check_bvh4(const Bvh4Image &w, const BvhImage &b2, std::string *why)
{
    auto bad = [&](const std::string &m) { if (why) *why = m; return false; };
    if (b2.n_nodes == 0) return w.n_nodes == 0 ? true : bad("nodes without a binary tree");
    // every leaf entry of the binary tree: its link and six planes
    std::vector<std::pair<int32_t, std::array<float, 6>>> leaves;
    for (int nd = 0; nd < b2.n_nodes; nd++)
        for (int k = 0; k < 2; k++) {
            const float *o = &b2.nodes[16 * (size_t)nd];
            std::array<float, 6> pl;
            if (k == 0) pl = {o[0], o[1], o[2], o[3], o[8], o[9]};
            else pl = {o[4], o[5], o[6], o[7], o[10], o[11]};
            if (!(pl[0] <= pl[1])) continue;
            int32_t link;
            std::memcpy(&link, &o[12 + k], 4);
            if (link < 0) leaves.push_back({link, pl});
        }
    std::sort(leaves.begin(), leaves.end(), [](const auto &a, const auto &b) { return a.first < b.first; });
    std::vector<int32_t> seen_leaves;
    std::vector<char> seen(w.n_nodes, 0);
    std::vector<int> stack{0};
    seen[0] = 1;
    while (!stack.empty()) {
        const int nd = stack.back();
        stack.pop_back();
        const float *o = &w.nodes[32 * (size_t)nd];
        for (int i = 0; i < 4; i++) {
            int32_t link;
            std::memcpy(&link, &o[24 + i], 4);
            std::array<float, 6> pl = {o[i], o[4 + i], o[8 + i], o[12 + i], o[16 + i], o[20 + i]};
            if (link == 0x7fffffff) {
                for (float v : pl) if (!(v == INFINITY)) return bad("unused slot with a finite plane");
                continue;
            }
            if (link >= 0) {
                if (link >= w.n_nodes || seen[link]) return bad("internal link out of range or shared");
                seen[link] = 1;
                stack.push_back(link);
                continue;
            }
            auto it = std::lower_bound(leaves.begin(), leaves.end(), link,
                                       [](const auto &a, int32_t l) { return a.first < l; });
            if (it == leaves.end() || it->first != link) return bad("leaf not in the binary tree");
            if (it->second != pl) return bad("leaf box differs from the binary tree's");
            seen_leaves.push_back(link);
        }
    }
    for (int nd = 0; nd < w.n_nodes; nd++)
        if (!seen[nd]) return bad("unreachable node");
    std::sort(seen_leaves.begin(), seen_leaves.end());
    if (seen_leaves.size() != leaves.size()) return bad("leaf count differs from the binary tree's");
    for (size_t i = 0; i < leaves.size(); i++)
        if (seen_leaves[i] != leaves[i].first) return bad("a leaf is reached twice or never");
    return true;
}

bool check_bvh2(const BvhImage &img, const float *tv, int n, int *depth, std::string *why)
{
    auto bad = [&](const std::string &m) { if (why) *why = m; return false; };
    if (n <= 0) { if (depth) *depth = 0; return img.n_nodes == 0 || bad("nodes for an empty scene"); }
    if (img.n_nodes <= 0 || img.n_slots != n) return bad("node or slot count");
    // every triangle must lie inside the boxes of all links on its path
    struct Item { int32_t link; int depth; int parent; };   // parent: index into boxes of the link's box
    std::vector<float> boxes;                                 // 6 floats per visited link
    std::vector<int> up;                                      // parent box of each box
    std::vector<Item> todo;
    std::vector<char> seen_slot(n, 0), seen_node(img.n_nodes, 0);
    const float *N0 = &img.nodes[0];
    auto push_children = [&](int node, int d, int parent) {
        const float *o = N0 + 16 * (size_t)node;
        int32_t l[2];
        std::memcpy(&l[0], &o[12], 4);
        std::memcpy(&l[1], &o[13], 4);
        const float b[2][6] = {{o[0], o[1], o[2], o[3], o[8], o[9]}, {o[4], o[5], o[6], o[7], o[10], o[11]}};
        for (int c = 0; c < 2; c++) {
            if (b[c][0] > b[c][1]) continue;   // empty second child of a root leaf
            int bi = (int)up.size();
            boxes.insert(boxes.end(), b[c], b[c] + 6);
            up.push_back(parent);
            todo.push_back({l[c], d + 1, bi});
        }
    };
    if (img.max_depth < 0) return bad("negative depth");
    int maxd = 0;
    seen_node[0] = 1;
    push_children(0, 0, -1);
    while (!todo.empty()) {
        Item it = todo.back();
        todo.pop_back();
        if (it.link >= 0) {
            if (it.link >= img.n_nodes || seen_node[it.link]) return bad("node linked twice or out of range");
            seen_node[it.link] = 1;
            push_children(it.link, it.depth, it.parent);
            continue;
        }
        maxd = std::max(maxd, it.depth);
        int v = ~it.link, first = v >> 3, cnt = (v & 7) + 1;
        if (first < 0 || first + cnt > n) return bad("leaf range out of slots");
        for (int k = first; k < first + cnt; k++) {
            if (seen_slot[k]) return bad("slot in two leaves");
            seen_slot[k] = 1;
            int32_t id;
            std::memcpy(&id, &img.tri_slots[12 * (size_t)k + 3], 4);
            if (id < 0 || id >= n) return bad("slot names no triangle");
            const float *p = tv + 9 * (size_t)id;
            for (int b = it.parent; b >= 0; b = up[b]) {
                const float *x = &boxes[6 * (size_t)b];
                for (int q = 0; q < 3; q++)
                    for (int a = 0; a < 3; a++)
                        if (!(p[3 * q + a] >= x[2 * a] && p[3 * q + a] <= x[2 * a + 1])) return bad("triangle outside a box");
            }
        }
    }
    for (int k = 0; k < n; k++) if (!seen_slot[k]) return bad("slot in no leaf");
    for (int k = 0; k < img.n_nodes; k++) if (!seen_node[k]) return bad("unreachable node");
    // the root leaf case reports depth 1 here (it hangs below a synthetic node)
    if (depth) *depth = maxd;
    return true;
}

}  // namespace rtgpu
