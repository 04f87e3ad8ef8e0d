// Internal structures shared by the C ABI (api.cu) and the kernel files.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "dshape.cuh"

namespace bgpu {

// leaf slot flags (third float4 .z of a slot, as int bits)
enum : int { SLOT_LAST = 1, SLOT_SHAPE = 2 };

// Device view of a scene's acceleration structure.  One of three node layouts
// (bvh.h) is resident:
//   binary (wide == 0): nodes, 4 float4 per inner node, root_ref
//   wide   (wide == 1): nodes8, 5 uint4 per 8-wide quantised node, root8
//   slots: 3 float4 per leaf slot, in the resident layout's leaf order:
//     triangle: (p1.xyz, e1.x) (e1.yz, e2.xy) (e2.z, prim, flags, 0)
//               with e1 = p2 - p1, e2 = p3 - p1 rounded exactly as the
//               reference computes them (TriangleMesh.hs:157-158, 169)
//     shape:    (shape index, 0, 0, 0) (0...) (0, prim, flags|SLOT_SHAPE, 0)
//   compact (wide == 2): nodesC, 2 float4 (32 bytes) per quantised binary
//     node, rootC
struct DevAccel {
  const float4* nodes;
  const uint4* nodes8;
  const float4* slots;
  const DShape* shapes;
  int32_t root_ref;
  int32_t root8;
  int32_t wide;  // node layout: 0 binary, 1 8-wide, 2 compact binary
  int32_t n_shapes;
  int64_t n_prims;
  const float4* nodesC;
  int32_t rootC;
  int32_t pad;
};

// node layouts (DevAccel::wide), the traversal's LAYOUT template argument
enum : int { LAYOUT_BINARY = 0, LAYOUT_WIDE = 1, LAYOUT_COMPACT = 2 };

// calls f(std::integral_constant<int, L>()) with L the node layout `layout`,
// to pick a kernel instantiation on the host
template <class F>
inline auto withLayout(int layout, F&& f) {
  switch (layout) {
    case LAYOUT_WIDE: return f(std::integral_constant<int, LAYOUT_WIDE>());
    case LAYOUT_COMPACT: return f(std::integral_constant<int, LAYOUT_COMPACT>());
    default: return f(std::integral_constant<int, LAYOUT_BINARY>());
  }
}

// Launchers (kernels_trace.cu); all enqueue on `stream` and return the
// launch status.  The persistent kernels take the next ray from *d_counter,
// which the launcher zeroes first (one counter per stream at a time).
cudaError_t launch_trace_closest(const DevAccel& A, const float* d_rays, int64_t n, float* d_t,
                                 int32_t* d_prim, float* d_b1b2, unsigned long long* d_counter,
                                 cudaStream_t stream);
// instrumented closest-hit traversal: adds node visits and leaf-slot tests
// into d_totals[0..1]
cudaError_t launch_trace_counts(const DevAccel& A, const float* d_rays, int64_t n,
                                unsigned long long* d_totals, cudaStream_t stream);
cudaError_t launch_trace_any(const DevAccel& A, const float* d_rays, int64_t n, uint8_t* d_hit,
                             unsigned long long* d_counter, cudaStream_t stream);

}  // namespace bgpu
