// bvh.h — binned-SAH BVH over triangles, flattened for the device.
//
// The reference's builder was never written (src/lib.rs is empty; the
// `ordered-float` dependency at Cargo.toml:19 hints at a sorted SAH). This
// builder bins centroids (32 bins, 3 axes; Wald 2007, "On fast Construction of
// SAH-based Bounding Volume Hierarchies") into a binary tree, then collapses
// it into a four-wide tree: every wide node takes a binary node's two
// children and keeps opening the inner child of largest surface area until it
// holds four (the collapse of Wald, Benthin and Boulos 2008, "Getting Rid of
// Packets"). One node fetch then tests four boxes, halving the chain of
// dependent node loads a ray walks.
//
// Device node layout: 128 bytes = eight 16-byte words, the four children's
// boxes side by side (slot k in component k of each word):
//   w0 = lo.x   w1 = hi.x   w2 = lo.y   w3 = hi.y   w4 = lo.z   w5 = hi.z
//   w6 = (child0, child1, child2, child3) as int32
//   w7 = (count0, count1, count2, count3) as int32 (not read by the kernels)
// child >= 0: index of an inner node. child < 0: leaf; ~child = first << 3 |
// count, the leaf's triangles being tri_order[first .. first + count) (count
// <= kBvhMaxLeaf <= 7). A node with fewer than four children fills the rest
// with empty slots: box lo = hi = +inf on every axis (missed by every ray) and
// child = ~0, a leaf of no triangles. Node 0 is the root; nodes are numbered
// depth first, children in slot order.
//
// Quantized node layout (the same tree, 64 bytes = four 16-byte words; after
// Ylitie, Karras and Laine 2017, "Efficient Incoherent Ray Traversal on
// GPUs Through Compressed Wide BVHs"): the children's boxes as 8-bit
// offsets in a per-node frame,
//   q0 = (origin.xyz as float, exponents ex | ey << 8 | ez << 16)
//   q1 = (child0..3 as int32, the same links as w6)
//   q2 = (qlo.x, qhi.x, qlo.y, qhi.y), q3 = (qlo.z, qhi.z, counts, 0), each
//        a 32-bit word holding one byte per child (child k in byte k).
// A plane decodes as fmaf(q, 2^(e - 127), origin) in float; the builder picks
// every q so that the decoded box contains the child's box (it evaluates the
// same fmaf), so a ray that hits a child's box hits its decoded box and the
// walk finds the same closest hit. Empty slots have child = ~0 and are
// skipped by the link, not by the box. Counts byte k = leaf size of child k.
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
constexpr int kBvhWidth = 4;
constexpr int kBvhNodeFloats = 32;   // 128-byte node
constexpr int kBvhQNodeFloats = 16;  // 64-byte quantized node
constexpr int kBvhStackSize = 96;    // traversal stack entries per ray

struct FlatBvh {
    std::vector<float> nodes;        // kBvhNodeFloats per node
    std::vector<int32_t> tri_order;  // leaf order -> scene triangle index
    int depth = 0;                   // wide nodes on the longest root-leaf path
    int max_leaf = 0;
    int max_stack = 0;               // most stack entries a traversal can hold
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // scene bounds
    int num_nodes() const { return (int)(nodes.size() / kBvhNodeFloats); }
};

// verts: 9 floats per triangle.
FlatBvh build_bvh(const float* verts, size_t num_tris);

// The quantized copy of a built tree, kBvhQNodeFloats per node (same node
// numbering and links).
std::vector<float> quantize_bvh(const FlatBvh& bvh);

}  // namespace aq
