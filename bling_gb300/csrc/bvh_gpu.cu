// BVH construction on the GPU (BLING_FLAG_GPU_BVH).
//
// Replaces the reference's kd-tree build (Primitive/KdTree.hs:81-203) for
// scenes that must become traceable quickly (admission of serving jobs,
// batches of freshly generated scenes).  The tree only has to contain every
// primitive: traversal is conservative and ties go to the larger primitive
// ID, so hit results do not depend on it.  Steps, all on the scene's stream:
//
//   1. centroid bounds                 k_centroid_bounds (block reductions)
//   2. 30-bit Morton code per centroid  k_morton
//   3. stable LSD radix sort of (code, primitive) pairs, 8 bits per pass
//                                      k_rs_hist / k_scan_* / k_rs_scatter
//   4. PLOC clustering (Meister and Bittner, "Parallel Locally-Ordered
//      Clustering for Bounding Volume Hierarchy Construction", 2018): the
//      Morton-ordered clusters each find the cluster within 16 positions
//      whose merged box has the smallest surface area; mutual nearest
//      neighbours merge into a new inner node, the rest move on; repeat
//      until one cluster is left.       k_ploc_nn / k_ploc_flag / k_ploc_merge
//   5. the inner nodes are written straight into the binary traversal layout
//      (64 bytes: both children's boxes, two child references; bvh.h) as they
//      are created; leaves hold one primitive each, in Morton order.
//
// Every step is deterministic: node indices come from prefix sums, not
// atomics, so a scene always gets the same tree.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>

#include "bvh.h"
#include "bvh_gpu.h"

namespace bgpu {
namespace {

constexpr int kRsThreads = 256;
constexpr int kRsItems = 16;                      // elements per thread per block
constexpr int kRsTile = kRsThreads * kRsItems;    // 4096 elements per block
constexpr int kRsBins = 256;
constexpr int kScanThreads = 1024;
constexpr int kPlocRadius = 16;

// ---------------------------------------------------------------- helpers
unsigned gridFor(int64_t n, int block, unsigned cap) {
  int64_t g = (n + block - 1) / block;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, cap));
}

// float <-> order-preserving unsigned (for atomicMin/atomicMax on floats)
__device__ __forceinline__ uint32_t fOrd(float f) {
  uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fUnord(uint32_t o) {
  uint32_t b = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
  return __uint_as_float(b);
}

// surface area of a box (lo.xyz, hi.xyz); empty extents count as zero
__device__ __forceinline__ float boxArea(float4 lo, float4 hi) {
  float dx = fmaxf(0.0f, hi.x - lo.x), dy = fmaxf(0.0f, hi.y - lo.y), dz = fmaxf(0.0f, hi.z - lo.z);
  return 2.0f * (dx * dy + dx * dz + dy * dz);
}

// spreads the low 10 bits of v to every third bit
__device__ __forceinline__ uint32_t spread10(uint32_t v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

// ---------------------------------------------------------------- 1, 2
// bounds of the primitive-box centroids: 6 ordered uints (min xyz, max xyz)
__global__ void __launch_bounds__(256) k_centroid_bounds(const float* __restrict__ lo,
                                                         const float* __restrict__ hi, int64_t n,
                                                         uint32_t* __restrict__ out) {
  float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    for (int a = 0; a < 3; a++) {
      float c = 0.5f * (lo[3 * i + a] + hi[3 * i + a]);
      mn[a] = fminf(mn[a], c);
      mx[a] = fmaxf(mx[a], c);
    }
  for (int a = 0; a < 3; a++)
    for (int o = 16; o > 0; o >>= 1) {
      mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
      mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
    }
  if ((threadIdx.x & 31) == 0)
    for (int a = 0; a < 3; a++) {
      atomicMin(out + a, fOrd(mn[a]));
      atomicMax(out + 3 + a, fOrd(mx[a]));
    }
}

__global__ void __launch_bounds__(256) k_morton(const float* __restrict__ lo,
                                                const float* __restrict__ hi, int64_t n,
                                                const uint32_t* __restrict__ cb,
                                                uint32_t* __restrict__ keys,
                                                int32_t* __restrict__ vals) {
  float mn[3], sc[3];
  for (int a = 0; a < 3; a++) {
    mn[a] = fUnord(cb[a]);
    float ext = fUnord(cb[3 + a]) - mn[a];
    sc[a] = ext > 0 ? 1023.0f / ext : 0.0f;
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t q[3];
    for (int a = 0; a < 3; a++) {
      float c = 0.5f * (lo[3 * i + a] + hi[3 * i + a]);
      float u = (c - mn[a]) * sc[a];
      u = fminf(fmaxf(u, 0.0f), 1023.0f);  // NaN -> 0
      q[a] = (uint32_t)u;
    }
    keys[i] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
    vals[i] = (int32_t)i;
  }
}

// ---------------------------------------------------------------- 3
// digit histogram of each block's tile: hist[digit * nblocks + block]
__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const uint32_t* __restrict__ keys,
                                                        int64_t n, int shift,
                                                        uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[kRsBins];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kRsTile;
  for (int k = 0; k < kRsItems; k++) {
    int64_t i = base + (int64_t)k * kRsThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xffu], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// exclusive prefix sum of a[0, count) in place, one block; *total = the sum
__global__ void __launch_bounds__(kScanThreads) k_scan_inplace(uint32_t* __restrict__ a,
                                                               int64_t count,
                                                               uint32_t* __restrict__ total) {
  __shared__ uint32_t warp_sums[kScanThreads / 32];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t base = 0; base < count; base += kScanThreads) {
    int64_t i = base + threadIdx.x;
    uint32_t v = i < count ? a[i] : 0u;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t s = warp_sums[lane];
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      warp_sums[lane] = s;  // inclusive over warps
    }
    __syncthreads();
    uint32_t excl = carry + (warp > 0 ? warp_sums[warp - 1] : 0u) + x - v;
    if (i < count) a[i] = excl;
    __syncthreads();
    if (threadIdx.x == kScanThreads - 1) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

// stable scatter of one block's tile by digit.  Elements are taken in
// rounds of kRsThreads consecutive elements; within a round a warp ranks
// its 32 elements per digit (__match_any_sync), the warps' digit counts are
// prefix-summed in shared memory, and the block's running count per digit
// carries over to the next round, so equal digits keep their input order.
__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(
    const uint32_t* __restrict__ kin, const int32_t* __restrict__ vin,
    uint32_t* __restrict__ kout, int32_t* __restrict__ vout, int64_t n, int shift,
    const uint32_t* __restrict__ hist_scanned) {
  constexpr int W = kRsThreads / 32;
  __shared__ uint32_t s_base[kRsBins];
  __shared__ uint32_t s_warp[W][kRsBins];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  s_base[threadIdx.x] = hist_scanned[(size_t)threadIdx.x * gridDim.x + blockIdx.x];
  const int64_t tile = (int64_t)blockIdx.x * kRsTile;
  for (int k = 0; k < kRsItems; k++) {
    for (int w = 0; w < W; w++) s_warp[w][threadIdx.x] = 0;
    __syncthreads();
    int64_t i = tile + (int64_t)k * kRsThreads + threadIdx.x;
    bool valid = i < n;
    uint32_t key = valid ? kin[i] : 0u;
    int32_t val = valid ? vin[i] : 0;
    uint32_t d = valid ? ((key >> shift) & 0xffu) : 0x100u;  // invalid lanes form their own group
    unsigned peers = __match_any_sync(0xffffffffu, d);
    unsigned rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && rank == 0) s_warp[warp][d] = __popc(peers);
    __syncthreads();
    // per digit: exclusive prefix over the warps, then the round's total
    {
      uint32_t acc = 0;
      for (int w = 0; w < W; w++) {
        uint32_t c = s_warp[w][threadIdx.x];
        s_warp[w][threadIdx.x] = acc;
        acc += c;
      }
      __syncthreads();
      if (valid) {
        uint32_t pos = s_base[d] + s_warp[warp][d] + rank;
        if (pos < n) {  // always, for a consistent histogram
          kout[pos] = key;
          vout[pos] = val;
        }
      }
      __syncthreads();
      s_base[threadIdx.x] += acc;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- 4, 5
// cluster arrays: box (lo, hi) as two float4 (w unused), node reference
// (>= 0 inner node, < 0 leaf ~slot) and subtree height
struct Clusters {
  float4* lo;
  float4* hi;
  int32_t* ref;
  int32_t* height;
};

__global__ void __launch_bounds__(256) k_ploc_init(const float* __restrict__ lo,
                                                   const float* __restrict__ hi,
                                                   const int32_t* __restrict__ order, int64_t n,
                                                   Clusters c) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int32_t p = order[i];
    c.lo[i] = make_float4(lo[3 * p], lo[3 * p + 1], lo[3 * p + 2], 0.0f);
    c.hi[i] = make_float4(hi[3 * p], hi[3 * p + 1], hi[3 * p + 2], 0.0f);
    c.ref[i] = ~(int32_t)i;  // leaf: slot i holds the i-th primitive in Morton order
    c.height[i] = 0;
  }
}

// nearest neighbour of every cluster within kPlocRadius positions: the one
// whose merged box has the smallest area (ties: the smaller position)
__global__ void __launch_bounds__(256) k_ploc_nn(Clusters c, int64_t m, int32_t* __restrict__ nn) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    float4 l = c.lo[i], h = c.hi[i];
    float best = INFINITY;
    int64_t bj = i == 0 ? 1 : i - 1;
    int64_t j0 = i - kPlocRadius < 0 ? 0 : i - kPlocRadius;
    int64_t j1 = i + kPlocRadius >= m ? m - 1 : i + kPlocRadius;
    for (int64_t j = j0; j <= j1; j++) {
      if (j == i) continue;
      float4 l2 = __ldg(&c.lo[j]), h2 = __ldg(&c.hi[j]);
      float a = boxArea(make_float4(fminf(l.x, l2.x), fminf(l.y, l2.y), fminf(l.z, l2.z), 0.0f),
                        make_float4(fmaxf(h.x, h2.x), fmaxf(h.y, h2.y), fmaxf(h.z, h2.z), 0.0f));
      if (a < best) {  // strict: the first (smallest) position wins ties
        best = a;
        bj = j;
      }
    }
    nn[i] = (int32_t)bj;
  }
}

// merge[i] = 1 for the lower position of a mutual pair (it makes the node);
// keep[i] = 0 for the higher position (its cluster joins the node)
__global__ void __launch_bounds__(256) k_ploc_flag(const int32_t* __restrict__ nn, int64_t m,
                                                   uint32_t* __restrict__ merge,
                                                   uint32_t* __restrict__ keep) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t j = nn[i];
    bool mutual = nn[j] == i;
    merge[i] = (mutual && i < j) ? 1u : 0u;
    keep[i] = (mutual && i > j) ? 0u : 1u;
  }
}

// writes the merged nodes (binary layout, bvh.h) and the next cluster array
__global__ void __launch_bounds__(256) k_ploc_merge(Clusters c, Clusters out, int64_t m,
                                                    const int32_t* __restrict__ nn,
                                                    const uint32_t* __restrict__ merge_pos,
                                                    const uint32_t* __restrict__ keep_pos,
                                                    const uint32_t* __restrict__ merge_flag,
                                                    const uint32_t* __restrict__ keep_flag,
                                                    int64_t node_base, int64_t node_cap,
                                                    float4* __restrict__ nodes) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (!keep_flag[i]) continue;
    int64_t p = keep_pos[i];
    if (p >= m) continue;  // never, for consistent prefix sums
    if (!merge_flag[i]) {
      out.lo[p] = c.lo[i];
      out.hi[p] = c.hi[i];
      out.ref[p] = c.ref[i];
      out.height[p] = c.height[i];
      continue;
    }
    int64_t j = nn[i];
    float4 l0 = c.lo[i], h0 = c.hi[i], l1 = c.lo[j], h1 = c.hi[j];
    int64_t node = node_base + merge_pos[i];
    if (node >= node_cap) continue;  // never: n - 1 merges in all
    float4* nd = nodes + 4 * node;
    nd[0] = make_float4(l0.x, h0.x, l0.y, h0.y);
    nd[1] = make_float4(l1.x, h1.x, l1.y, h1.y);
    nd[2] = make_float4(l0.z, h0.z, l1.z, h1.z);
    nd[3] = make_float4(__int_as_float(c.ref[i]), __int_as_float(c.ref[j]), 0.0f, 0.0f);
    out.lo[p] = make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), 0.0f);
    out.hi[p] = make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.0f);
    out.ref[p] = (int32_t)node;
    out.height[p] = 1 + max(c.height[i], c.height[j]);
  }
}

#define GB_CUDA(call)                                                         \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      err = std::string("GPU BVH build: ") + #call + ": " + cudaGetErrorString(e_); \
      return e_ == cudaErrorMemoryAllocation ? -2 : -3;                       \
    }                                                                         \
  } while (0)

// per block of kScanTile elements: exclusive prefix sums in place and the
// block's total in sums[block]
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) k_scan_partial(uint32_t* __restrict__ a,
                                                               int64_t count,
                                                               uint32_t* __restrict__ sums) {
  __shared__ uint32_t warp_sums[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t t = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    v[k] = base + k < count ? a[base + k] : 0u;
    t += v[k];
  }
  uint32_t x = t;  // inclusive scan of the thread totals over the warp
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = warp_sums[lane];
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    warp_sums[lane] = w;
  }
  __syncthreads();
  uint32_t run = (warp > 0 ? warp_sums[warp - 1] : 0u) + x - t;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < count) a[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = warp_sums[31];
}

__global__ void __launch_bounds__(256) k_scan_add(uint32_t* __restrict__ a, int64_t count,
                                                  const uint32_t* __restrict__ sums) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] += sums[i / kScanTile];
}

// exclusive prefix sum of a[0, count) in place (count < 2^31; sums holds
// count / kScanTile + 1 words); the total goes to *d_total
cudaError_t scanInplace(uint32_t* a, int64_t count, uint32_t* sums, uint32_t* d_total,
                        unsigned cap, cudaStream_t s) {
  if (count <= kScanTile) {
    k_scan_inplace<<<1, kScanThreads, 0, s>>>(a, count, d_total);
    return cudaGetLastError();
  }
  const int64_t nb = (count + kScanTile - 1) / kScanTile;
  k_scan_partial<<<(unsigned)nb, kScanThreads, 0, s>>>(a, count, sums);
  k_scan_inplace<<<1, kScanThreads, 0, s>>>(sums, nb, d_total);
  k_scan_add<<<gridFor(count, 256, cap), 256, 0, s>>>(a, count, sums);
  return cudaGetLastError();
}

}  // namespace

void GpuBvh::release() {
  cudaFree(nodes);
  cudaFree(order);
  nodes = nullptr;
  order = nullptr;
}

int build_bvh_gpu(cudaStream_t s, const float* d_lo, const float* d_hi, int64_t n, GpuBvh& out,
                  std::string& err) {
  out = GpuBvh{};
  if (n <= 0 || n >= (int64_t(1) << 27)) {
    err = "GPU BVH build: primitive count out of range";
    return -1;
  }
  int dev = 0, sms = 1;
  GB_CUDA(cudaGetDevice(&dev));
  GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const unsigned cap = (unsigned)sms * 16u;
  const int64_t nblocks = (n + kRsTile - 1) / kRsTile;
  // scratch: keys and values twice, histogram, 6 bound words, counters,
  // clusters twice, nn, flags and positions
  size_t b_keys = sizeof(uint32_t) * n, b_vals = sizeof(int32_t) * n;
  size_t b_hist = sizeof(uint32_t) * kRsBins * nblocks;
  size_t b_cl = (2 * sizeof(float4) + 2 * sizeof(int32_t)) * n;
  size_t b_sums = sizeof(uint32_t) * (std::max<int64_t>(kRsBins * nblocks, n) / kScanTile + 2);
  size_t total = 2 * b_keys + 2 * b_vals + b_hist + 64 + 2 * b_cl + sizeof(int32_t) * n +
                 4 * sizeof(uint32_t) * n + b_sums + 24 * 256;  // + rounding of 24 arrays
  unsigned char* scratch = nullptr;
  GB_CUDA(cudaMalloc(&scratch, total));
  auto fail = [&](int rc) {
    cudaFree(scratch);
    out.release();
    return rc;
  };
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char* p = scratch + off;
    off += (bytes + 255) / 256 * 256;
    return p;
  };
  uint32_t* k0 = (uint32_t*)take(b_keys);
  uint32_t* k1 = (uint32_t*)take(b_keys);
  int32_t* v0 = (int32_t*)take(b_vals);
  int32_t* v1 = (int32_t*)take(b_vals);
  uint32_t* hist = (uint32_t*)take(b_hist);
  uint32_t* words = (uint32_t*)take(64);  // centroid bounds [0, 6), scan totals [8, 10)
  Clusters ca, cb;
  ca.lo = (float4*)take(sizeof(float4) * n);
  ca.hi = (float4*)take(sizeof(float4) * n);
  ca.ref = (int32_t*)take(sizeof(int32_t) * n);
  ca.height = (int32_t*)take(sizeof(int32_t) * n);
  cb.lo = (float4*)take(sizeof(float4) * n);
  cb.hi = (float4*)take(sizeof(float4) * n);
  cb.ref = (int32_t*)take(sizeof(int32_t) * n);
  cb.height = (int32_t*)take(sizeof(int32_t) * n);
  int32_t* nn = (int32_t*)take(sizeof(int32_t) * n);
  uint32_t* mflag = (uint32_t*)take(sizeof(uint32_t) * n);
  uint32_t* kflag = (uint32_t*)take(sizeof(uint32_t) * n);
  uint32_t* mpos = (uint32_t*)take(sizeof(uint32_t) * n);
  uint32_t* kpos = (uint32_t*)take(sizeof(uint32_t) * n);
  uint32_t* sums = (uint32_t*)take(sizeof(uint32_t) * (std::max(kRsBins * nblocks, n) / kScanTile + 2));
  if (off > total) {  // the layout above must fit the allocation
    err = "GPU BVH build: scratch layout overflow";
    return fail(-3);
  }
  cudaError_t e;
#define GB_STEP(call)                                                          \
  do {                                                                         \
    if ((e = (call)) != cudaSuccess) {                                         \
      err = std::string("GPU BVH build: ") + #call + ": " + cudaGetErrorString(e); \
      return fail(e == cudaErrorMemoryAllocation ? -2 : -3);                   \
    }                                                                          \
  } while (0)

  // 1, 2: centroid bounds and Morton codes
  uint32_t init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
  GB_STEP(cudaMemcpyAsync(words, init, sizeof init, cudaMemcpyHostToDevice, s));
  k_centroid_bounds<<<gridFor(n, 256, cap), 256, 0, s>>>(d_lo, d_hi, n, words);
  k_morton<<<gridFor(n, 256, cap), 256, 0, s>>>(d_lo, d_hi, n, words, k0, v0);
  GB_STEP(cudaGetLastError());
  // 3: radix sort, 8 bits per pass (the codes have 30 bits: four passes)
  for (int shift = 0; shift < 32; shift += 8) {
    k_rs_hist<<<(unsigned)nblocks, kRsThreads, 0, s>>>(k0, n, shift, hist);
    GB_STEP(cudaGetLastError());
    GB_STEP(scanInplace(hist, (int64_t)kRsBins * nblocks, sums, words + 8, cap, s));
    k_rs_scatter<<<(unsigned)nblocks, kRsThreads, 0, s>>>(k0, v0, k1, v1, n, shift, hist);
    GB_STEP(cudaGetLastError());
    std::swap(k0, k1);
    std::swap(v0, v1);
  }
  // the primitive order of the leaf slots (Morton order)
  GB_STEP(cudaMalloc(&out.order, sizeof(int32_t) * n));
  GB_STEP(cudaMemcpyAsync(out.order, v0, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
  out.n_prims = n;
  if (n == 1) {  // a single leaf
    out.root_ref = ~0;
    out.depth = 0;
    GB_STEP(cudaStreamSynchronize(s));
    cudaFree(scratch);
    return 0;
  }
  // 4: PLOC, writing inner nodes as they are made
  GB_STEP(cudaMalloc(&out.nodes, sizeof(float4) * 4 * (n - 1)));
  k_ploc_init<<<gridFor(n, 256, cap), 256, 0, s>>>(d_lo, d_hi, out.order, n, ca);
  GB_STEP(cudaGetLastError());
  int64_t m = n, made = 0;
  int iterations = 0;
  while (m > 1) {
    if (++iterations > 100000) {  // each round merges at least one pair
      err = "GPU BVH build: clustering did not converge";
      return fail(-3);
    }
    unsigned g = gridFor(m, 256, cap);
    k_ploc_nn<<<g, 256, 0, s>>>(ca, m, nn);
    k_ploc_flag<<<g, 256, 0, s>>>(nn, m, mflag, kflag);
    GB_STEP(cudaGetLastError());
    GB_STEP(cudaMemcpyAsync(mpos, mflag, sizeof(uint32_t) * m, cudaMemcpyDeviceToDevice, s));
    GB_STEP(cudaMemcpyAsync(kpos, kflag, sizeof(uint32_t) * m, cudaMemcpyDeviceToDevice, s));
    GB_STEP(scanInplace(mpos, m, sums, words + 8, cap, s));
    GB_STEP(scanInplace(kpos, m, sums, words + 9, cap, s));
    k_ploc_merge<<<g, 256, 0, s>>>(ca, cb, m, nn, mpos, kpos, mflag, kflag, made, n - 1,
                                   out.nodes);
    GB_STEP(cudaGetLastError());
    uint32_t tot[2];
    GB_STEP(cudaMemcpyAsync(tot, words + 8, sizeof tot, cudaMemcpyDeviceToHost, s));
    GB_STEP(cudaStreamSynchronize(s));
    if (tot[0] == 0 || (int64_t)tot[1] != m - (int64_t)tot[0]) {
      err = "GPU BVH build: inconsistent clustering round";
      return fail(-3);
    }
    made += tot[0];
    m = tot[1];
    std::swap(ca, cb);
  }
  if (made != n - 1) {
    err = "GPU BVH build: wrong inner node count";
    return fail(-3);
  }
  int32_t root = 0, height = 0;
  GB_STEP(cudaMemcpyAsync(&root, ca.ref, sizeof root, cudaMemcpyDeviceToHost, s));
  GB_STEP(cudaMemcpyAsync(&height, ca.height, sizeof height, cudaMemcpyDeviceToHost, s));
  GB_STEP(cudaStreamSynchronize(s));
  out.root_ref = root;
  out.depth = height;
  out.n_nodes = n - 1;
  out.iterations = iterations;
  cudaFree(scratch);
  return 0;
#undef GB_STEP
}

}  // namespace bgpu

namespace bgpu {
namespace {
__global__ void __launch_bounds__(256) k_gather_slots(const float4* __restrict__ src,
                                                      const int32_t* __restrict__ order, int64_t n,
                                                      float4* __restrict__ dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t s = i / 3, k = i - 3 * s;
    dst[i] = src[3 * (int64_t)order[s] + k];
  }
}
}  // namespace

cudaError_t launch_gather_slots(const float4* src, const int32_t* order, int64_t n, float4* dst,
                                cudaStream_t stream) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_gather_slots<<<gridFor(3 * n, 256, (unsigned)sms * 16u), 256, 0, stream>>>(src, order, n, dst);
  return cudaGetLastError();
}

}  // namespace bgpu
