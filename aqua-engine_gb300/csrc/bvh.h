// bvh.h — binned-SAH BVH over triangles, flattened for the device.
//
// The reference's builder was never written (src/lib.rs is empty; the
// `ordered-float` dependency at Cargo.toml:19 hints at a sorted SAH). This
// builder bins centroids (32 bins, 3 axes; Wald 2007, "On fast Construction of
// SAH-based Bounding Volume Hierarchies") and writes a two-wide node array the
// traversal kernels read with 128-bit loads.
//
// Device node layout: 64 bytes = four 16-byte words, both children's boxes in
// the parent so one node fetch tests two boxes.
//   w0 = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   w1 = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   w2 = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   w3 = (child0, child1, count0, count1) as int32
// child >= 0: index of an inner node. child < 0: leaf; ~child = first << 3 |
// count, the leaf's triangles being tri_order[first .. first + count) (count
// <= kBvhMaxLeaf <= 7; the count is repeated in count0/count1). Node 0 is the
// root.
//
// Triangle layout (leaf order): three 16-byte words per triangle,
//   t0 = (v0.xyz, scene index as int bits)
//   t1 = (v1.xyz, material | (light + 1) << 16 as int bits)
//   t2 = (v2.xyz, 0)
#pragma once

#include <stdint.h>

#include <vector>

namespace aq {

constexpr int kBvhMaxLeaf = 4;
constexpr int kBvhMaxDepth = 64;  // traversal stack bound

struct FlatBvh {
    std::vector<float> nodes;        // 16 floats per node
    std::vector<int32_t> tri_order;  // leaf order -> scene triangle index
    int depth = 0;
    int max_leaf = 0;
    int num_nodes() const { return (int)(nodes.size() / 16); }
};

// verts: 9 floats per triangle.
FlatBvh build_bvh(const float* verts, size_t num_tris);

}  // namespace aq
