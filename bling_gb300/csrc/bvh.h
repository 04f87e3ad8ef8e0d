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
};

// Returns 0 on success, -1 if the input is empty/invalid.
int build_bvh(const BvhBuildInput& in, BvhBuildOutput& out);

// Depth bound honoured by the builder; traversal stacks are sized from it.
constexpr int kBvhMaxDepth = 60;

}  // namespace bgpu
