// Ray-query kernels: one thread per ray over SoA ray buffers.
#include "internal.h"
#include "trace.cuh"

namespace bgpu {

__device__ __forceinline__ Ray loadRay(const float* __restrict__ rays, int64_t n, int64_t i) {
  return Ray{V3{__ldg(rays + i), __ldg(rays + n + i), __ldg(rays + 2 * n + i)},
             V3{__ldg(rays + 3 * n + i), __ldg(rays + 4 * n + i), __ldg(rays + 5 * n + i)},
             __ldg(rays + 6 * n + i), __ldg(rays + 7 * n + i)};
}

__global__ void k_trace_closest(DevAccel A, const float* __restrict__ rays, int64_t n,
                                float* __restrict__ out_t, int32_t* __restrict__ out_prim,
                                float* __restrict__ out_b) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Ray r = loadRay(rays, n, i);
  float t, b1, b2;
  int prim;
  bool hit = traverse<false>(A, r, t, prim, b1, b2);
  out_t[i] = hit ? t : INFINITY;
  out_prim[i] = hit ? prim : -1;
  if (out_b) {
    out_b[2 * i] = b1;
    out_b[2 * i + 1] = b2;
  }
}

__global__ void k_trace_any(DevAccel A, const float* __restrict__ rays, int64_t n,
                            uint8_t* __restrict__ out_hit) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Ray r = loadRay(rays, n, i);
  float t, b1, b2;
  int prim;
  out_hit[i] = traverse<true>(A, r, t, prim, b1, b2) ? 1 : 0;
}

__global__ void k_trace_counts(DevAccel A, const float* __restrict__ rays, int64_t n,
                               unsigned long long* __restrict__ totals) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  TraversalCounts c{0, 0};
  if (i < n) {
    Ray r = loadRay(rays, n, i);
    float t, b1, b2;
    int prim;
    traverse<false, true>(A, r, t, prim, b1, b2, &c);
  }
  // warp reduction, one atomic per warp
  for (int o = 16; o > 0; o >>= 1) {
    c.nodes += __shfl_down_sync(0xffffffffu, c.nodes, o);
    c.slots += __shfl_down_sync(0xffffffffu, c.slots, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(totals, (unsigned long long)c.nodes);
    atomicAdd(totals + 1, (unsigned long long)c.slots);
  }
}

cudaError_t launch_trace_counts(const DevAccel& A, const float* d_rays, int64_t n,
                                unsigned long long* d_totals, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  int64_t grid = (n + 127) / 128;
  k_trace_counts<<<(unsigned)grid, 128, 0, stream>>>(A, d_rays, n, d_totals);
  return cudaGetLastError();
}

cudaError_t launch_trace_closest(const DevAccel& A, const float* d_rays, int64_t n, float* d_t,
                                 int32_t* d_prim, float* d_b1b2, int block, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  if (block <= 0) block = 128;
  int64_t grid = (n + block - 1) / block;
  k_trace_closest<<<(unsigned)grid, block, 0, stream>>>(A, d_rays, n, d_t, d_prim, d_b1b2);
  return cudaGetLastError();
}

cudaError_t launch_trace_any(const DevAccel& A, const float* d_rays, int64_t n, uint8_t* d_hit,
                             int block, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  if (block <= 0) block = 128;
  int64_t grid = (n + block - 1) / block;
  k_trace_any<<<(unsigned)grid, block, 0, stream>>>(A, d_rays, n, d_hit);
  return cudaGetLastError();
}

}  // namespace bgpu
