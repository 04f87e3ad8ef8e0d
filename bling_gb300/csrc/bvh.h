// Host-side BVH construction for the GPU traversal kernels.
//
// Replaces the reference's kd-tree build (Primitive/KdTree.hs:107-203): an
// exact-event SAH kd-tree with primitives referenced from several leaves.
// The GPU instead gets a binary BVH built with a binned surface-area
// heuristic over primitive centroids, each primitive in exactly one leaf, laid
// out as 64-byte nodes (both children's boxes plus two child references) in
// depth-first order.  Only the hit results have to match the reference;
// traversal order is free, and ties are resolved by primitive ID.
#pragma once
#include <cstdint>
#include <vector>

namespace bgpu {

struct BvhBuildInput {
  int64_t n = 0;                // primitives, in primitive-ID order
  const float* lo = nullptr;    // 3n: world-space box minimum per primitive
  const float* hi = nullptr;    // 3n: box maximum
  int max_leaf = 4;             // primitives per leaf at most (when splittable)
  int threads = 0;              // 0: hardware concurrency
  bool wide = true;             // also produce the 8-wide quantised layout
  bool compact = false;         // also produce the 32-byte quantised binary layout
};

struct BvhBuildOutput {
  // 16 floats per internal node:
  //   [0..3]  child0 lo.x hi.x lo.y hi.y
  //   [4..7]  child1 lo.x hi.x lo.y hi.y
  //   [8..11] child0 lo.z hi.z, child1 lo.z hi.z
  //   [12..13] child refs (int bits): >= 0 internal node, < 0 leaf whose first
  //            slot is ~ref; [14..15] unused
  std::vector<float> nodes;
  std::vector<int32_t> slot_prim;   // primitive ID per leaf slot, leaf order
  std::vector<uint8_t> slot_last;   // 1 on the last slot of each leaf
  int32_t root_ref = 0;             // like a child ref
  int max_depth = 0;
  int64_t leaves = 0;

  // The same tree collapsed to 8-wide nodes with 8-bit quantised child boxes
  // (filled when BvhBuildInput::wide).  20 words (80 bytes) per node:
  //   w0: origin p.xyz (float), biased exponents ex|ey<<8|ez<<16 (scale 2^(e-127))
  //   w1: first internal child node, first leaf slot, meta[0..3], meta[4..7]
  //       meta: 0x80|rank internal child (node child_base + rank),
  //             offset of a leaf child's first slot from the slot base, 0xFF empty
  //   w2..w4: qlo.x[8] qlo.y[8] | qlo.z[8] qhi.x[8] | qhi.y[8] qhi.z[8]
  // child box = p + q * scale, widened by one quantum where possible.
  // Child slots are ordered so that visiting slot k ^ octant(ray) for
  // k = 0..7 is roughly front to back.  The leaf slots follow a different
  // order than the binary layout's, so they come in their own arrays.
  std::vector<uint32_t> nodes8;
  std::vector<int32_t> slot_prim8;
  std::vector<uint8_t> slot_last8;
  int32_t root8 = 0;      // node 0, or a leaf ref when the whole scene is one leaf
  int wide_depth = 0;     // longest root-to-leaf path in wide nodes

  // The binary tree in 32-byte quantised nodes (filled when
  // BvhBuildInput::compact), one 256-bit load per visit.  8 words per node:
  //   w0..w2  origin p.xyz (float): the node's box minimum
  //   w3      biased exponents ex | ey << 8 | ez << 16 (scale 2^(e - 127)),
  //           meta << 24: bit 0 child 0 is a leaf, bit 1 child 1 is a leaf,
  //           bits 2..7 the slot count of a leaf child 0
  //   w4..w6  child boxes q, bytes: c0 lo.xyz hi.xyz, c1 lo.xyz hi.xyz
  //           (box = p + q * scale, rounded outward by one quantum)
  //   w7      both children inner: child 1's node (child 0 is the next node);
  //           otherwise the first slot of leaf child 0; a leaf child 1's
  //           slots follow it, an inner child 1 is the next node
  // Nodes are in depth-first order and a node with one leaf child keeps it
  // as child 0, so one word locates both children.  The leaf slots follow
  // their own order.
  std::vector<uint32_t> nodesC;
  std::vector<int32_t> slot_primC;
  std::vector<uint8_t> slot_lastC;
  int32_t rootC = 0;      // node 0, or a leaf ref when the whole scene is one leaf
  bool compact_ok = false;
};

constexpr int kWideStack = 128;  // per-lane stack entries of the wide traversal

// Returns 0 on success, -1 if the input is empty/invalid.
int build_bvh(const BvhBuildInput& in, BvhBuildOutput& out);

// Structural check of a built tree against the primitive boxes: every
// primitive is in exactly one leaf slot of each layout, slots end with a
// SLOT_LAST flag, every inner box contains its children and every decoded
// quantised child box contains the child (exact arithmetic).  Returns 0, or a
// negative code naming the first violation.
int validate_bvh(const BvhBuildInput& in, const BvhBuildOutput& out);

// Depth bound honoured by the builder; traversal stacks are sized from it.
constexpr int kBvhMaxDepth = 60;

}  // namespace bgpu
