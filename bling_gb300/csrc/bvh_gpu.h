// BVH construction on the GPU (bvh_gpu.cu): Morton order, PLOC clustering,
// the binary 64-byte node layout of bvh.h with one primitive per leaf.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace bgpu {

struct GpuBvh {
  float4* nodes = nullptr;   // 4 float4 per inner node (bvh.h's binary layout); n - 1 nodes
  int32_t* order = nullptr;  // primitive of leaf slot i (Morton order); n entries
  int32_t root_ref = 0;      // inner node index, or ~0 when the scene is one primitive
  int depth = 0;             // edges on the longest root-to-leaf path
  int iterations = 0;        // clustering rounds
  int64_t n_nodes = 0, n_prims = 0;
  void release();            // frees nodes and order
};

// Builds the tree of n primitive boxes (d_lo/d_hi: 3n floats each, device
// memory, primitive-ID order) on `stream`; synchronises it.  Returns 0, or a
// negative code with a message (-2 out of device memory, -1 bad input,
// -3 a CUDA error or an inconsistent clustering round).
int build_bvh_gpu(cudaStream_t stream, const float* d_lo, const float* d_hi, int64_t n,
                  GpuBvh& out, std::string& err);

// dst[3 i + k] = src[3 order[i] + k] for k < 3 (leaf slots, 48 bytes each,
// gathered from primitive order into leaf order)
cudaError_t launch_gather_slots(const float4* src, const int32_t* order, int64_t n, float4* dst,
                                cudaStream_t stream);

}  // namespace bgpu
