// Ray-query kernels over SoA ray buffers: persistent warps (trace.cuh,
// traceWarpPersistent), one instantiation per node layout, plus the
// instrumented variant that counts the traversal work.
#include <algorithm>

#include "internal.h"
#include "trace.cuh"

namespace bgpu {

__device__ __forceinline__ Ray loadRay(const float* __restrict__ rays, int64_t n, int64_t i) {
  return Ray{V3{__ldg(rays + i), __ldg(rays + n + i), __ldg(rays + 2 * n + i)},
             V3{__ldg(rays + 3 * n + i), __ldg(rays + 4 * n + i), __ldg(rays + 5 * n + i)},
             __ldg(rays + 6 * n + i), __ldg(rays + 7 * n + i)};
}

constexpr int kTraceBlock = 128;
static_assert(kTraceBlock <= kMaxTraceBlock, "the traversal's shared stack holds kMaxTraceBlock lanes");

template <int LAYOUT>
__global__ void __launch_bounds__(kTraceBlock)
    k_trace_closest(DevAccel A, const float* __restrict__ rays, int64_t n,
                    float* __restrict__ out_t, int32_t* __restrict__ out_prim,
                    float* __restrict__ out_b, unsigned long long* __restrict__ next_ray) {
  traceWarpPersistent<false, LAYOUT, false>(
      A, n, next_ray, [&](int64_t i) { return loadRay(rays, n, i); },
      [&](int64_t i, const RayQueryResult& q) {
        out_t[i] = q.hit ? q.t : INFINITY;
        out_prim[i] = q.hit ? q.prim : -1;
        if (out_b) {
          out_b[2 * i] = q.b1;
          out_b[2 * i + 1] = q.b2;
        }
      });
}

template <int LAYOUT>
__global__ void __launch_bounds__(kTraceBlock, 10)
    k_trace_any(DevAccel A, const float* __restrict__ rays, int64_t n,
                uint8_t* __restrict__ out_hit, unsigned long long* __restrict__ next_ray) {
  traceWarpPersistent<true, LAYOUT, false>(
      A, n, next_ray, [&](int64_t i) { return loadRay(rays, n, i); },
      [&](int64_t i, const RayQueryResult& q) { out_hit[i] = q.hit ? 1 : 0; });
}

// totals[0] nodes visited, totals[1] leaf slots tested, totals[2] the next-ray counter
template <int LAYOUT>
__global__ void __launch_bounds__(kTraceBlock)
    k_trace_counts(DevAccel A, const float* __restrict__ rays, int64_t n,
                   unsigned long long* __restrict__ totals) {
  TraversalCounts c{0, 0};
  traceWarpPersistent<false, LAYOUT, true>(
      A, n, totals + 2, [&](int64_t i) { return loadRay(rays, n, i); },
      [&](int64_t, const RayQueryResult&) {}, &c);
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

// resident blocks for a persistent launch: SMs x blocks per SM at full occupancy
template <class K>
static unsigned persistentGrid(K kernel, int64_t n) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTraceBlock, 0);
  int64_t g = (int64_t)std::max(1, sms) * std::max(1, per_sm);
  int64_t need = (n + kTraceBlock - 1) / kTraceBlock;
  return (unsigned)std::max<int64_t>(1, std::min(g, need));
}

cudaError_t launch_trace_counts(const DevAccel& A, const float* d_rays, int64_t n,
                                unsigned long long* d_totals, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(d_totals, 0, 3 * sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return e;
  return withLayout(A.wide, [&](auto L) {
    constexpr int LY = decltype(L)::value;
    k_trace_counts<LY><<<persistentGrid(k_trace_counts<LY>, n), kTraceBlock, 0, stream>>>(
        A, d_rays, n, d_totals);
    return cudaGetLastError();
  });
}

cudaError_t launch_trace_closest(const DevAccel& A, const float* d_rays, int64_t n, float* d_t,
                                 int32_t* d_prim, float* d_b1b2, unsigned long long* d_counter,
                                 cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return e;
  return withLayout(A.wide, [&](auto L) {
    constexpr int LY = decltype(L)::value;
    k_trace_closest<LY><<<persistentGrid(k_trace_closest<LY>, n), kTraceBlock, 0, stream>>>(
        A, d_rays, n, d_t, d_prim, d_b1b2, d_counter);
    return cudaGetLastError();
  });
}

cudaError_t launch_trace_any(const DevAccel& A, const float* d_rays, int64_t n, uint8_t* d_hit,
                             unsigned long long* d_counter, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return e;
  return withLayout(A.wide, [&](auto L) {
    constexpr int LY = decltype(L)::value;
    k_trace_any<LY><<<persistentGrid(k_trace_any<LY>, n), kTraceBlock, 0, stream>>>(
        A, d_rays, n, d_hit, d_counter);
    return cudaGetLastError();
  });
}

}  // namespace bgpu
