// rt_bvh.h -- host-side acceleration-structure build for the device tracer.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace rtgpu {

// Deepest leaf of a built tree (root at depth 0).  The BVH2 traversals keep
// one stack entry per level plus a sentinel in 64 entries (RT_STACK), so the
// builder bounds the depth at 62 (see Builder::build).
#define RT_BVH_DEPTH_CAP 62

// Device BVH2 image.  Each internal node is 4 float4 (64 bytes):
//   n0 = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   n1 = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   n2 = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   n3 = (child0, child1, 0, 0) as int32: >= 0 internal node index,
//        < 0 leaf, ~c = (first_slot << 3) | (count - 1), count <= 8.
// Leaf triangles occupy consecutive slots of 3 float4 each:
//   (p0.xyz, tri id bits), (e1.xyz, 0), (e2.xyz, 0) with e1 = p1 - p0,
//   e2 = p2 - p0 computed in binary32 exactly as Triangle::intersection
//   forms them (geometricShape/Triangle.cpp:51-52).
struct BvhImage {
    std::vector<float> nodes;      // 16 floats per node
    std::vector<float> tri_slots;  // 12 floats per slot
    int n_nodes = 0;
    int n_slots = 0;
    int max_depth = 0;
    double sah_cost = 0.0;
};

// 4-wide BVH collapsed from a BVH2 image; it shares the BVH2's triangle
// slots and leaf encoding.  Each node is 8 float4 (128 bytes, one cache
// line), one plane of the four child boxes per float4:
//   xlo[4], xhi[4], ylo[4], yhi[4], zlo[4], zhi[4], link[4] (int32), pad
// link >= 0: internal node; < 0: leaf as in the BVH2.  An unused slot has
// every plane at +inf, a box no ray can enter whatever its direction.  The
// child boxes are the BVH2's (already widened), so the 4-wide traversal
// culls exactly what the BVH2's would.
struct Bvh4Image {
    std::vector<float> nodes;      // 32 floats per node
    std::vector<int32_t> src;      // per node and slot: the BVH2 child it copies (node * 2 + child), -1 unused
    int n_nodes = 0;
    int max_depth = 0;             // deepest node level below the root
};

// Collapse a BVH2 image: every 4-wide node takes the two children of a
// binary node and opens the internal child of largest surface area until it
// has four children (or only leaves).
void build_bvh4(const BvhImage &b2, Bvh4Image &out);
// Structural check of a 4-wide image against the BVH2 it was collapsed
// from: every node reached once, every BVH2 leaf reached exactly once with
// the BVH2's box, unused slots all +inf.
bool check_bvh4(const Bvh4Image &w, const BvhImage &b2, std::string *why);

// A binary tree built elsewhere (the reference's SAH BVH, flattened to one
// tree over the scene's triangles), as topology only: node i is internal
// when count == 0 (children left and right), else a leaf over
// prims[first, first + count) (triangle indices).  Node 0 is the root.
struct ExtNode { int32_t left, right, first, count; };

// The BVH2 image of such a tree: every node reached once, every triangle in
// exactly one leaf; boxes are recomputed from the triangles (and widened as
// build_bvh2 widens them), and leaves of more than 8 triangles are split in
// halves of their range.  False with a reason when the tree is malformed or
// deeper than depth_cap.
bool import_bvh2(const float *tri_v, int n_tris, const ExtNode *nodes, int n_nodes, const int32_t *prims,
                 int n_prims, BvhImage &out, std::string *why, int depth_cap = RT_BVH_DEPTH_CAP);

// Compressed 8-wide BVH.  Each node is 5 float4 (80 bytes):
//   w0 = (px, py, pz, bits: ex | ey << 8 | ez << 16)      grid origin, exponents
//   w1 = (child_base, tri_base, meta[0..3], meta[4..7])   as int32 / packed bytes
//   w2 = (qlo.x[0..7], qlo.y[0..7])   w3 = (qlo.z[0..7], qhi.x[0..7])
//   w4 = (qhi.y[0..7], qhi.z[0..7])   one byte per child slot
// Child box = p + q * 2^(e-127) per axis, quantised outward.  meta[i]:
//   0 empty; 0xE0 | k internal child node child_base + k;
//   (c << 5) | k leaf of c in 1..3 triangles at slots tri_base + k.
// Slot i holds the child reached first by rays whose direction signs are the
// bits of i (bit a set: negative along axis a); a ray with sign bits o visits
// the slots in the order k ^ o, k = 0..7.
struct WideBvhImage {
    std::vector<float> nodes;      // 20 floats per node
    std::vector<float> tri_slots;  // 12 floats per slot, same layout as BvhImage
    int n_nodes = 0;
    int n_slots = 0;
    int max_depth = 0;
};

// Build from triangle vertex positions (9 floats per triangle).  Boxes are
// widened outward by a few ulps so the fused slab test never culls a node
// that contains a hit the exact Moller-Trumbore test accepts.
// c_node: the SAH cost of visiting a node, in units of one triangle test
// depth_cap: deepest leaf level allowed (object-median splits below it)
void build_bvh2(const float *tri_v, int n_tris, BvhImage &out, int max_leaf = 4, int n_bins = 32,
                double c_node = 1.0, int depth_cap = RT_BVH_DEPTH_CAP);

// Binned-SAH binary tree (leaves of at most 3 triangles) collapsed into the
// compressed 8-wide layout above, greedily opening the child of largest
// surface area until a node has 8 children.
void build_wbvh8(const float *tri_v, int n_tris, WideBvhImage &out, int n_bins = 32,
                 int depth_cap = RT_BVH_DEPTH_CAP);

// Structural check of a BVH2 image against its triangles: every node reached
// once, every triangle in exactly one leaf and inside the box of every link
// on its path.  Reports the deepest leaf below the root node (links count as
// levels); false with a reason otherwise.
bool check_bvh2(const BvhImage &img, const float *tri_v, int n_tris, int *depth, std::string *why);

}  // namespace rtgpu
