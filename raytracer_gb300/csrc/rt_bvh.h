// rt_bvh.h -- host-side acceleration-structure build for the device tracer.
#pragma once
#include <cstdint>
#include <vector>

namespace rtgpu {

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

// Build from triangle vertex positions (9 floats per triangle).  Boxes are
// widened outward by a few ulps so the fused slab test never culls a node
// that contains a hit the exact Moller-Trumbore test accepts.
void build_bvh2(const float *tri_v, int n_tris, BvhImage &out, int max_leaf = 4, int n_bins = 32);

}  // namespace rtgpu
