// Host SAH BVH builder and the device layout it produces.
//
// Replaces the reference's acceleration structure (OCTree,
// src/tracer/accel/octree.cpp:7-51,135-151) with a binned-SAH binary BVH,
// flattened to 64-byte nodes that hold both children's boxes (one 4 x float4
// load per visited node) and a triangle array in leaf order (3 x float4 per
// triangle: the exact vertices, so the device Moller-Trumbore test computes
// the same edges as the reference, mesh.cpp:186-187).
#pragma once

#include <cstdint>
#include <vector>

namespace dl {

// 64-byte node, 16-byte aligned: the boxes of both children.
//   a = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   b = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   c = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   d = (child0, child1, 0, 0) as int bits
// child >= 0: index of an inner node; child < 0: leaf ~((first << 4) | (count - 1)),
// first = index of the first triangle in the leaf-ordered triangle array,
// count in [1, 16].  Both slots of every node hold a child (a one-leaf tree
// references its leaf twice); only the root of an empty tree holds kEmptyRef
// (with inverted boxes), and the traversal never visits it.
struct alignas(16) GpuNode {
    float a[4];
    float b[4];
    float c[4];
    int32_t d[4];
};
static_assert(sizeof(GpuNode) == 64, "node layout");

// 48-byte triangle: v0.xyz + original triangle id (int bits), v1.xyz +
// material type of its mesh (set by the scene), v2.xyz + 0.
struct alignas(16) GpuTri {
    float v0[3];
    int32_t prim;
    float v1[3];
    int32_t mat_type;
    float v2[3];
    int32_t pad2;
};
static_assert(sizeof(GpuTri) == 48, "triangle layout");

constexpr int32_t kEmptyRef = 0x7fffffff;  // child slot without a subtree
constexpr int kMaxLeafTris = 16;
constexpr int kMaxDepth = 60;      // build depth cap; traversal stack holds 64 entries
constexpr int kTraversalStack = 64;

struct BvhBuildOptions {
    int max_leaf_size = 4;         // SAH leaves hold at most this many triangles
    int bins = 32;
    float traversal_cost = 1.0f;
    float intersect_cost = 0.5f;   // a triangle test costs half a node visit (both child
                                   // boxes) in the traversal kernels: measured best of 0.25-2
    int threads = 0;               // 0 = hardware concurrency
};

struct BvhResult {
    std::vector<GpuNode> nodes;    // nodes[0] is the root (always an inner node)
    std::vector<GpuTri> tris;      // leaf order
    std::vector<int32_t> tri_order; // leaf-order index -> original triangle id
    int depth = 0;
    int leaves = 0;
    double sah_cost = 0.0;
    double seconds = 0.0;
};

// tris: n x 9 floats (p0, p1, p2), original order.
BvhResult build_bvh(const float* tris, int64_t n, const BvhBuildOptions& opt);

}  // namespace dl
