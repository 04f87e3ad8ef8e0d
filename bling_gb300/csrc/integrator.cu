// Wavefront path integrator on the GPU.
//
// One pass of the reference's sampler renderer (prender/tile,
// Rendering.hs:111-150) with the path integrator (Integrator/Path.hs:30-87):
// every pixel of the filter-padded sample extent gets strata_x*strata_y
// camera paths.  Paths live in SoA slots (throughput and radiance as 16-band
// spectra, band-major) and never move; queues of slot indices carry the live
// paths from stage to stage.  Each bounce (one vertex of every live path,
// nextVertex, Path.hs:49-87) is five launches:
//
//   k_trace         closest hit of the bounce rays (scIntersect), and each
//                   path's shading class, which k_class_scatter sorts by
//   k_shade         emission on specular paths, the BSDF, one light sample and
//                   one BSDF sample for MIS (sampleOneLight/estimateDirect,
//                   Scene.hs:61-118), Russian roulette and the continuation
//                   sample; queues the shadow ray, the MIS ray and the vertex
//   k_trace_shadow  any hit of the shadow rays (occluded), and the MIS rays'
//                   occlusion queries (wavefront.cuh, occlusionSlot)
//   k_resolve       adds the vertex's radiance, updates the throughput,
//                   queues the continuing paths and splats finished ones into
//                   the film (addSample, Image.hs:250-299)
//
// The three traversal launches are persistent warps (trace.cuh); queues are
// appended with one atomic per warp (__ballot_sync/__popc).  Arithmetic keeps
// the reference's operation order (-fmad=false), random numbers come from the
// counter-based generator shared with the CPU oracle.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "filter_host.h"
#include "wavefront.cuh"

namespace bgpu {

// the pass's 16x16 filter table and the ray-binning counters sit between
// the counters and the slots
constexpr size_t kFilterBytes = 256 * sizeof(float);
constexpr int kRayBinBits = 15;  // direction octant (3 bits) x 16^3 origin cells
constexpr int kRayBins = 1 << kRayBinBits;
constexpr size_t kRayBinBytes = kRayBins * sizeof(unsigned);

// lays counters, the filter table, the bin counters, slots and queues out in
// one buffer of slotBytes(cap) bytes
static size_t slotBytes(size_t cap) {
  return kCounterBytes + kFilterBytes + kRayBinBytes + (kSlotWords + kQueueWords) * 4 * cap;
}

static void carve(unsigned char* base, size_t cap, Slots& st, Queues& q,
                  unsigned long long*& counters, float*& filter, unsigned*& bins) {
  counters = (unsigned long long*)base;
  filter = (float*)(base + kCounterBytes);
  bins = (unsigned*)(base + kCounterBytes + kFilterBytes);
  float* w = (float*)(base + kCounterBytes + kFilterBytes + kRayBinBytes);
  carveSlots(w, cap, st);
  int32_t* qw = (int32_t*)w;
  q.live[0] = qw;
  q.live[1] = qw + cap;
  q.shadow = qw + 2 * cap;  // 2 cap entries: shadow rays and MIS rays
  q.resolve = qw + 4 * cap;
  q.sorted = qw + 5 * cap;
  q.cls = qw + 6 * cap;
}

__device__ __forceinline__ unsigned* classCounts(unsigned long long* counters) {
  return (unsigned*)counters + kClassCountsAt;
}

// ------------------------------------------------------------------ kernels
// camera rays (fireRay, Camera.hs:49-68) for samples [chunk_base, chunk_base + count)
__global__ void k_raygen(PassParams P, bling_camera_desc cam, Slots st, int64_t count,
                         int32_t* __restrict__ queue, unsigned long long* counters) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    Ray ray = cameraRay(P, cam, P.chunk_base + (uint64_t)i);
    storeRay(st.ray, (int)i, ray);
    storeBands(st.T, (int)i, sConst(1.0f));
    storeBands(st.L, (int)i, sConst(0.0f));
    queue[i] = (int32_t)i;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) counters[C_LIVE0] = (unsigned long long)count;
}

// zeroes the per-bounce counters and the next live queue's size
__global__ void k_bounce_reset(unsigned long long* counters, int next_live) {
  int t = threadIdx.x;
  if (t == 0) counters[next_live] = 0;
  if (t == 1) counters[C_NEXT_TRACE] = 0;
  if (t == 2) counters[C_SHADOW] = 0;
  if (t == 4) counters[C_RESOLVE] = 0;
  if (t == 5) counters[C_NEXT_SHADOW] = 0;
  if (t < 32) classCounts(counters)[t] = 0;  // class counts [0, 16) and cursors [16, 32)
}

// the live queue in shading-class order: each block ranks its entries per
// class in shared memory (warp-aggregated), then reserves one range per class
// present with a single global atomic
__global__ void __launch_bounds__(128) k_class_scatter(const int32_t* __restrict__ queue,
                                                       const unsigned long long* __restrict__ qcount,
                                                       const int32_t* __restrict__ cls,
                                                       int32_t* __restrict__ sorted,
                                                       unsigned long long* __restrict__ counters) {
  __shared__ unsigned off[kShadeClasses];
  __shared__ unsigned s_cnt[kShadeClasses], s_base[kShadeClasses];
  classOffsets(classCounts(counters), off);
  unsigned* cursor = classCounts(counters) + 16;
  int64_t n = (int64_t)*qcount;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t nround = (n + stride - 1) / stride * stride;  // the same trip count in every thread
  const int lane = threadIdx.x & 31;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nround; q += stride) {
    if (threadIdx.x < kShadeClasses) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    int c = q < n ? cls[q] : -1;
    unsigned grp = __match_any_sync(0xffffffffu, c);
    int leader = __ffs(grp) - 1;
    unsigned wbase = 0;
    if (c >= 0 && lane == leader) wbase = atomicAdd(s_cnt + c, (unsigned)__popc(grp));
    wbase = __shfl_sync(0xffffffffu, wbase, leader);
    __syncthreads();
    if (threadIdx.x < kShadeClasses && s_cnt[threadIdx.x])
      s_base[threadIdx.x] = atomicAdd(cursor + threadIdx.x, s_cnt[threadIdx.x]);
    __syncthreads();
    if (c >= 0) sorted[off[c] + s_base[c] + wbase + __popc(grp & ((1u << lane) - 1))] = queue[q];
    __syncthreads();  // s_cnt and s_base are rewritten by the next trip
  }
}

// ---- ray binning (BLING_FLAG_BIN_RAYS): a bounce's live queue in the order
// of (direction octant, Morton code of the origin's cell in a 16^3 grid over
// the scene's bounds), so that the rays of a warp start near one another and
// head the same way and share the BVH nodes they fetch.  A counting sort: one
// counting pass (keys kept in the queue's class array, which is free until
// the shading sort), a scan and a scatter.  Order within a bin is arbitrary;
// it only changes which warp traces a ray.
struct BinFrame {
  float lo[3], scale[3];  // cell = (o - lo) * scale, clamped to [0, 15]
};

__device__ __forceinline__ uint32_t spread4(uint32_t v) {  // 4 bits -> every third bit
  return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4) | ((v & 8u) << 6);
}

__device__ __forceinline__ uint32_t rayBinKey(const Ray& r, const BinFrame& F) {
  const float o[3] = {r.o.x, r.o.y, r.o.z}, d[3] = {r.d.x, r.d.y, r.d.z};
  uint32_t cell = 0, oct = 0;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    float u = (o[a] - F.lo[a]) * F.scale[a];
    u = fminf(fmaxf(u, 0.0f), 15.0f);  // NaN -> 0
    cell |= spread4((uint32_t)u) << a;
    oct |= (signbit(d[a]) ? 1u : 0u) << a;
  }
  return (oct << 12) | cell;
}

__global__ void __launch_bounds__(128) k_raybin_count(Slots st, const int32_t* __restrict__ queue,
                                                      const unsigned long long* __restrict__ qcount,
                                                      BinFrame F, int32_t* __restrict__ keys,
                                                      unsigned* __restrict__ bins) {
  const int64_t n = (int64_t)*qcount;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t nround = (n + stride - 1) / stride * stride;
  const int lane = threadIdx.x & 31;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nround; q += stride) {
    uint32_t key = 0xffffffffu;
    if (q < n) {
      key = rayBinKey(loadRay7(st.ray, queue[q]), F);
      keys[q] = (int32_t)key;
    }
    unsigned grp = __match_any_sync(0xffffffffu, key);  // one atomic per distinct key
    if (key != 0xffffffffu && lane == __ffs(grp) - 1) atomicAdd(bins + key, (unsigned)__popc(grp));
  }
}

// exclusive scan of the kRayBins counters in place (one block of 1024)
__global__ void __launch_bounds__(1024) k_raybin_scan(unsigned* __restrict__ bins) {
  __shared__ unsigned part[1024];
  constexpr int per = kRayBins / 1024;
  const int t = threadIdx.x;
  unsigned sum = 0;
  for (int k = 0; k < per; k++) sum += bins[t * per + k];
  part[t] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    unsigned v = t >= off ? part[t - off] : 0u;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  unsigned run = part[t] - sum;
  for (int k = 0; k < per; k++) {
    unsigned v = bins[t * per + k];
    bins[t * per + k] = run;
    run += v;
  }
}

__global__ void __launch_bounds__(128) k_raybin_scatter(const int32_t* __restrict__ queue,
                                                        const unsigned long long* __restrict__ qcount,
                                                        const int32_t* __restrict__ keys,
                                                        unsigned* __restrict__ bins,
                                                        int32_t* __restrict__ out) {
  const int64_t n = (int64_t)*qcount;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t nround = (n + stride - 1) / stride * stride;
  const int lane = threadIdx.x & 31;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nround; q += stride) {
    uint32_t key = q < n ? (uint32_t)keys[q] : 0xffffffffu;
    unsigned grp = __match_any_sync(0xffffffffu, key);
    int leader = __ffs(grp) - 1;
    unsigned base = 0;
    if (key != 0xffffffffu && lane == leader) base = atomicAdd(bins + key, (unsigned)__popc(grp));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (key != 0xffffffffu) {
      unsigned pos = base + __popc(grp & ((1u << lane) - 1u));
      if ((int64_t)pos < n) out[pos] = queue[q];  // always, for consistent counts
    }
  }
}

// closest hit of the live paths' rays (scIntersect); as each ray finishes,
// its path's shading class goes to cls (by queue position) and is counted,
// per block in shared memory, then once per class and block
template <int LAYOUT>
__global__ void __launch_bounds__(128, 8) k_trace(DevAccel A, DevShading S, Slots st,
                                               const int32_t* __restrict__ queue,
                                               const unsigned long long* __restrict__ qcount,
                                               int32_t* __restrict__ cls,
                                               unsigned long long* __restrict__ counters) {
  __shared__ unsigned s_counts[kShadeClasses];
  if (threadIdx.x < kShadeClasses) s_counts[threadIdx.x] = 0;
  __syncthreads();
  int64_t n = (int64_t)*qcount;
  traceWarpPersistent<false, LAYOUT, false>(
      A, n, counters + C_NEXT_TRACE, [&](int64_t q) { return loadRay7(st.ray, queue[q]); },
      [&](int64_t q, const RayQueryResult& res) {
        float4 rec = hitRecord(res.hit, res.t, res.prim, res.b1, res.b2);
        st.hit[queue[q]] = rec;
        int c = shadeClass(A, S, __float_as_int(rec.y));
        cls[q] = c;
        atomicAdd(s_counts + c, 1u);
      });
  __syncthreads();  // every warp has left its walk
  if (threadIdx.x < kShadeClasses && s_counts[threadIdx.x])
    atomicAdd(classCounts(counters) + threadIdx.x, s_counts[threadIdx.x]);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(counters + C_CLOSEST, (unsigned long long)n);
}

// occlusion of the shadow rays (occluded, Scene.hs:45-47) and whether the
// MIS rays toward lights other than area lights hit anything
template <int LAYOUT>
__global__ void __launch_bounds__(128, 8) k_trace_shadow(DevAccel A, Slots st,
                                                      const int32_t* __restrict__ queue,
                                                      unsigned long long* __restrict__ counters) {
  int64_t n = (int64_t)counters[C_SHADOW];
  traceWarpPersistent<true, LAYOUT, false, true>(
      A, n, counters + C_NEXT_SHADOW,
      [&](int64_t q, bool& by_intersect, int& rank_prim) {
        return loadOcclusionRay(st, queue[q], by_intersect, rank_prim);
      },
      [&](int64_t q, const RayQueryResult& res) {
        storeOcclusion(st, queue[q], res, counters + C_DEGENERATE);
      });
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(counters + C_ANY, (unsigned long long)n);
}

// one vertex of every live path, up to its shadow and MIS rays (Path.hs:49-87)
template <bool TEX>
__global__ void __launch_bounds__(128, 4) k_shade(DevAccel A, DevShading S, PassParams P, Slots st,
                                               Queues Q, const int32_t* __restrict__ qin,
                                               int depth, int live_in,
                                               float* __restrict__ film, const float* filter,
                                               unsigned long long* __restrict__ counters) {
  // qin: the live paths in shading-class order
  int64_t n = (int64_t)counters[live_in];
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t nround = (n + stride - 1) / stride * stride;  // whole warps stay together for the appends
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nround; q += stride) {
    VertexOut o{false, false, false};
    int s = 0;
    if (q < n) {
      s = qin[q];
      uint64_t g = P.chunk_base + (uint64_t)s;  // slots never move
      o = shadeVertex<TEX>(A, S, P, st, s, g, depth, counters, [&](const Spec& L) {
        splatSample(film, P, g, L, counters, TableFilter{filter});
      });
    }
    queueAppend(o.shadow, s, Q.shadow, counters + C_SHADOW);
    queueAppend(o.mis, ~s, Q.shadow, counters + C_SHADOW);
    queueAppend(o.resolve, s, Q.resolve, counters + C_RESOLVE);
  }
}

// the vertex's radiance and the continuation (Path.hs:60-87)
__global__ void __launch_bounds__(128) k_resolve(DevAccel A, DevShading S, PassParams P, Slots st,
                                                 Queues Q, int live_out, float* __restrict__ film,
                                                 const float* filter,
                                                 unsigned long long* __restrict__ counters) {
  int64_t n = (int64_t)counters[C_RESOLVE];
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t nround = (n + stride - 1) / stride * stride;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nround; q += stride) {
    bool cont = false;
    int s = 0;
    if (q < n) {
      s = Q.resolve[q];
      uint64_t g = P.chunk_base + (uint64_t)s;
      Spec Tn, Ln;
      bool l_same = false;
      cont = resolveVertex<true>(
          A, S, st, s, counters,
          [&](const Spec& L) {
            splatSample(film, P, g, L, counters, TableFilter{filter});
          },
          Tn, Ln, &l_same);
      if (cont) {
        storeBands(st.T, s, Tn);
        if (!l_same) storeBands(st.L, s, Ln);
      }
    }
    queueAppend(cont, s, Q.live[live_out], counters + live_out);
  }
}

// ------------------------------------------------------------------ host side
namespace {

template <class K>
unsigned residentGrid(K kernel, int sms) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0);
  return (unsigned)(std::max(1, sms) * std::max(1, per_sm));
}

struct Grids {
  unsigned trace, shadow, shade, resolve, raygen;
};
Grids g_grids[64];
bool g_grids_ready[64] = {false};
std::mutex g_grids_mu;  // callers on any thread

Grids grids(int device, int sms) {
  std::lock_guard<std::mutex> lk(g_grids_mu);
  if (device >= 0 && device < 64 && g_grids_ready[device]) return g_grids[device];
  Grids g;
  // the layouts' kernels use the same registers within a few; take the smallest grid
  g.trace = std::min({residentGrid(k_trace<LAYOUT_BINARY>, sms), residentGrid(k_trace<LAYOUT_WIDE>, sms),
                      residentGrid(k_trace<LAYOUT_COMPACT>, sms)});
  g.shadow = std::min({residentGrid(k_trace_shadow<LAYOUT_BINARY>, sms),
                       residentGrid(k_trace_shadow<LAYOUT_WIDE>, sms),
                       residentGrid(k_trace_shadow<LAYOUT_COMPACT>, sms)});
  g.shade = residentGrid(k_shade<false>, sms);
  g.resolve = residentGrid(k_resolve, sms);
  g.raygen = (unsigned)std::max(1, sms * 8);
  if (device >= 0 && device < 64) {
    g_grids[device] = g;
    g_grids_ready[device] = true;
  }
  return g;
}


// the bounces of one chunk of path samples
cudaError_t runChunk(cudaStream_t stream, const DevAccel& A, const DevShading& S, PassParams P,
                     Slots st, Queues Q, unsigned long long* counters, int64_t count, int max_depth,
                     float* d_film, const float* d_filter, const Grids& G, unsigned* d_bins,
                     const BinFrame* bin) {
  const int block = 128;
  unsigned g_ray = (unsigned)std::min<int64_t>((count + block - 1) / block, (int64_t)G.raygen);
  k_raygen<<<g_ray, block, 0, stream>>>(P, S.camera, st, count, Q.live[0], counters);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  unsigned cap_blocks = (unsigned)std::max<int64_t>(1, (count + block - 1) / block);
  for (int depth = 0; depth <= max_depth; depth++) {
    int in = depth & 1;
    k_bounce_reset<<<1, 32, 0, stream>>>(counters, C_LIVE0 + (1 - in));
    unsigned gt = std::min(G.trace, cap_blocks), gs = std::min(G.shadow, cap_blocks);
    // the bounce's queue: binned into Q.sorted (bounces after the camera's,
    // whose rays are in pixel order already), then shading-class sorted into
    // whichever of the two queues is free
    const unsigned long long* qn = counters + C_LIVE0 + in;
    int32_t* traced = Q.live[in];
    int32_t* shaded = Q.sorted;
    if (bin && depth > 0) {
      cudaMemsetAsync(d_bins, 0, kRayBinBytes, stream);
      k_raybin_count<<<G.raygen, block, 0, stream>>>(st, Q.live[in], qn, *bin, Q.cls, d_bins);
      k_raybin_scan<<<1, 1024, 0, stream>>>(d_bins);
      k_raybin_scatter<<<G.raygen, block, 0, stream>>>(Q.live[in], qn, Q.cls, d_bins, Q.sorted);
      traced = Q.sorted;
      shaded = Q.live[in];
    }
    withLayout(A.wide, [&](auto L) {
      k_trace<decltype(L)::value><<<gt, block, 0, stream>>>(A, S, st, traced, qn, Q.cls, counters);
    });
    k_class_scatter<<<G.raygen, block, 0, stream>>>(traced, qn, Q.cls, shaded, counters);
    if (S.textured)
      k_shade<true><<<std::min(G.shade, cap_blocks), block, 0, stream>>>(
          A, S, P, st, Q, shaded, depth, C_LIVE0 + in, d_film, d_filter, counters);
    else
      k_shade<false><<<std::min(G.shade, cap_blocks), block, 0, stream>>>(
          A, S, P, st, Q, shaded, depth, C_LIVE0 + in, d_film, d_filter, counters);
    withLayout(A.wide, [&](auto L) {
      k_trace_shadow<decltype(L)::value><<<gs, block, 0, stream>>>(A, st, Q.shadow, counters);
    });
    k_resolve<<<std::min(G.resolve, cap_blocks), block, 0, stream>>>(A, S, P, st, Q,
                                                                      C_LIVE0 + (1 - in), d_film,
                                                                      d_filter, counters);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

// the pass constants (imageWindow', Image.hs:170-176; Path.hs:34-36)
int integrator_pass_params(const bling_render_params& p, uint64_t pass, int fw, int fh, PassParams& P,
               std::string& err) {
  memset(&P, 0, sizeof P);
  P.seed = p.seed;
  P.pass = pass;
  float fwid, fhei;
  if (p.filter_kind == BLING_FILTER_BOX) {
    fwid = fhei = 0.5f;
  } else {
    fwid = p.filter_params[0];
    fhei = p.filter_params[1];
  }
  if (!(fwid > 0) || !(fhei > 0) || fwid > 16 || fhei > 16) {
    err = "filter extent must be in (0, 16]";
    return BLING_ERR_INVALID_ARG;
  }
  P.fw = fwid;
  P.fh = fhei;
  P.x0 = (int)floorf(0.5f - fwid);
  P.x1 = (int)floorf(0.5f + (float)p.width + fwid);
  P.y0 = (int)floorf(0.5f - fhei);
  P.y1 = (int)floorf(0.5f + (float)p.height + fhei);
  P.nx = P.x1 - P.x0 + 1;
  P.ny = P.y1 - P.y0 + 1;
  P.nu = p.strata_x;
  P.nv = p.strata_y;
  P.spp = p.strata_x * p.strata_y;
  P.random = p.sampler_kind == BLING_SAMPLER_RANDOM ? 1 : 0;
  // stratified dimensions (Path.hs:34-36); the Random sampler has none, its
  // rnd'/rnd2D' always draw fresh uniforms (Sampling.hs:203-221)
  P.n1d = P.random ? 0 : 4 * p.sample_depth;
  P.n2d = P.random ? 0 : 3 * p.sample_depth;
  P.max_depth = p.max_depth;
  P.rr_depth = p.rr_depth;
  P.width = fw;
  P.height = fh;
  return BLING_OK;
}

#define RET_CUDA(call)                                                      \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) {                                                \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);             \
      return e_ == cudaErrorMemoryAllocation ? BLING_ERR_OOM : BLING_ERR_CUDA; \
    }                                                                       \
  } while (0)

void integrator_workspace_free(IntegratorWorkspace& ws) {
  cudaFree(ws.buffer);
  ws = IntegratorWorkspace{};
}

// A workspace of at least `cap` path slots, or, when the device has no room
// for that many, the largest of cap/2, cap/4, ... down to kMinWorkspaceSlots
// (the pass runs in more chunks then).  A workspace already holding at least
// the floor is kept when a larger one does not fit.
constexpr size_t kMinWorkspaceSlots = size_t(1) << 20;

static int ensureWorkspace(IntegratorWorkspace& ws, size_t cap, std::string& err) {
  if (ws.capacity >= cap && ws.buffer) return BLING_OK;
  const size_t floor_slots = std::min(cap, kMinWorkspaceSlots);
  for (size_t c = cap;; c = std::max(floor_slots, (c / 2 + 63) / 64 * 64)) {
    if (ws.buffer && ws.capacity >= c) return BLING_OK;  // the one we have is as large
    void* buf = nullptr;
    cudaError_t e = cudaMalloc(&buf, slotBytes(c));
    if (e == cudaSuccess) {
      integrator_workspace_free(ws);
      ws.buffer = buf;
      ws.capacity = c;
      return BLING_OK;
    }
    if (e != cudaErrorMemoryAllocation) RET_CUDA(e);
    (void)cudaGetLastError();  // clear the allocation error before trying smaller
    if (c == floor_slots) break;
  }
  if (ws.buffer && ws.capacity >= floor_slots) return BLING_OK;
  char buf[160];
  snprintf(buf, sizeof buf, "no device memory for a path workspace of %zu slots (%zu bytes)",
           floor_slots, slotBytes(floor_slots));
  err = buf;
  return BLING_ERR_OOM;
}

// the pixel and sample number of the lowest dropped sample index g, kept
// as ~g in C_FIRST_NONFINITE (decodeSample's order)
static void firstDropped(const PassParams& P, unsigned long long v, PassResult& res) {
  if (!v) return;
  uint64_t g = ~(uint64_t)v;
  uint64_t pix = g / (uint64_t)P.spp;
  res.nf_n = (int32_t)(g % (uint64_t)P.spp);
  res.nf_x = P.x0 + (int32_t)(pix % (uint64_t)P.nx);
  res.nf_y = P.y0 + (int32_t)(pix / (uint64_t)P.nx);
}

int integrator_render_pass(cudaStream_t stream, const DevAccel& A, const DevShading& S,
                           const bling_render_params& p, uint64_t pass, float* d_film, int fw,
                           int fh, IntegratorWorkspace& ws, PassResult& res, std::string& err,
                           const float* bin_box) {
  int device = 0;
  RET_CUDA(cudaGetDevice(&device));
  RET_CUDA(loadCieConstants(device));
  PassParams P;
  int rc = integrator_pass_params(p, pass, fw, fh, P, err);
  if (rc) return rc;
  uint64_t total = (uint64_t)P.nx * P.ny * P.spp;
  if (total >= (uint64_t(1) << 40)) {
    err = "too many samples in one pass";
    return BLING_ERR_INVALID_ARG;
  }
  size_t cap = (size_t)std::min<uint64_t>(total, uint64_t(1) << 24);
  // a multiple of 64 paths keeps every per-path array 16-byte aligned (the
  // records are read with 16-byte vector loads)
  cap = (std::max<size_t>(cap, 1024) + 63) / 64 * 64;
  rc = ensureWorkspace(ws, cap, err);
  if (rc) return rc;
  Slots st;
  Queues Q;
  unsigned long long* counters;
  float* d_filter;
  unsigned* d_bins;
  carve((unsigned char*)ws.buffer, ws.capacity, st, Q, counters, d_filter, d_bins);
  BinFrame frame;
  if (bin_box)
    for (int a = 0; a < 3; a++) {
      float ext = bin_box[3 + a] - bin_box[a];
      frame.lo[a] = bin_box[a];
      frame.scale[a] = ext > 0 ? 16.0f / ext : 0.0f;
    }
  float tbl[256];
  filterTableHost(p.filter_kind, p.filter_params, P.fw, P.fh, tbl);
  RET_CUDA(cudaMemcpyAsync(d_filter, tbl, sizeof tbl, cudaMemcpyHostToDevice, stream));
  RET_CUDA(cudaMemsetAsync(counters, 0, C_COUNT * sizeof(unsigned long long), stream));
  int sms = 0;
  RET_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  Grids G = grids(device, sms);
  for (uint64_t base = 0; base < total; base += ws.capacity) {
    int64_t count = (int64_t)std::min<uint64_t>(ws.capacity, total - base);
    P.chunk_base = base;
    RET_CUDA(runChunk(stream, A, S, P, st, Q, counters, count, p.max_depth, d_film, d_filter, G,
                      d_bins, bin_box ? &frame : nullptr));
  }
  unsigned long long cnt[C_COUNT];
  RET_CUDA(cudaMemcpyAsync(cnt, counters, sizeof cnt, cudaMemcpyDeviceToHost, stream));
  RET_CUDA(cudaStreamSynchronize(stream));
  res.rays_closest = cnt[C_CLOSEST];
  res.rays_any = cnt[C_ANY];
  res.nonfinite = cnt[C_NONFINITE];
  res.degenerate = cnt[C_DEGENERATE];
  res.path_samples = total;
  firstDropped(P, cnt[C_FIRST_NONFINITE], res);
  return BLING_OK;
}

// ------------------------------------------------------------------ no-allocation pass
// Path state for bling_render_pass_noalloc, in one file-scope device array:
// the wavefront of one pass of at most kNoAllocSlots path samples (counters,
// filter table, slots and queues, laid out by carve()).  Every GPU that loads
// the library holds it (about 35 MiB) until the process exits.  All calls
// share the array; the counters and the filter table are written at the
// start of every call and the path state is written before it is read.  Two
// calls whose work overlaps on the GPU (different streams or contexts on one
// device) race on it.
constexpr size_t kNoAllocSlots = size_t(1) << 16;
constexpr size_t kNoAllocBytes =
    kCounterBytes + kFilterBytes + kRayBinBytes + (kSlotWords + kQueueWords) * 4 * kNoAllocSlots;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {
constexpr int kMaxDevices = 64;
unsigned char* g_noalloc_ptr[kMaxDevices] = {nullptr};
std::mutex g_noalloc_mu;  // guards the per-device address table
}  // namespace

size_t integrator_noalloc_max_samples() { return kNoAllocSlots; }

int integrator_render_pass_noalloc(cudaStream_t stream, const DevAccel& A, const DevShading& S,
                                   const bling_render_params& p, uint64_t pass, float* d_film,
                                   int fw, int fh, PassResult& res, std::string& err) {
  int device = 0;
  RET_CUDA(cudaGetDevice(&device));
  if (device < 0 || device >= kMaxDevices) {
    err = "device ordinal out of range for the no-allocation pass";
    return BLING_ERR_INVALID_ARG;
  }
  // set-up, once per device with that device current: the host-side name of
  // a __device__ array is not a device address, so fetch the address
  unsigned char* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[device]) {
      void* ptr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess || !ptr) {
        err = std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e);
        return BLING_ERR_CUDA;
      }
      g_noalloc_ptr[device] = (unsigned char*)ptr;
    }
    scratch = g_noalloc_ptr[device];
  }
  // the film must be device memory of this device: a host pointer would fault
  // in the kernels
  {
    cudaPointerAttributes pa;
    cudaError_t e = cudaPointerGetAttributes(&pa, d_film);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      err = std::string("film pointer: ") + cudaGetErrorString(e);
      return BLING_ERR_INVALID_ARG;
    }
    if (pa.type != cudaMemoryTypeDevice && pa.type != cudaMemoryTypeManaged) {
      err = "the film must be device memory (cudaMalloc or managed), not a host pointer";
      return BLING_ERR_INVALID_ARG;
    }
    if (pa.device != device) {
      err = "the film lives on another device than the scene";
      return BLING_ERR_INVALID_ARG;
    }
  }
  RET_CUDA(loadCieConstants(device));
  PassParams P;
  int rc = integrator_pass_params(p, pass, fw, fh, P, err);
  if (rc) return rc;
  uint64_t total = (uint64_t)P.nx * P.ny * P.spp;
  if (total > kNoAllocSlots) {
    char buf[256];
    snprintf(buf, sizeof buf,
             "pass needs %llu path samples (%d x %d sample extent x %d strata); the "
             "no-allocation pass holds at most %llu",
             (unsigned long long)total, P.nx, P.ny, P.spp, (unsigned long long)kNoAllocSlots);
    err = buf;
    return BLING_ERR_BOUNDS;
  }
  Slots st;
  Queues Q;
  unsigned long long* counters;
  float* d_filter;
  unsigned* d_bins;
  carve(scratch, kNoAllocSlots, st, Q, counters, d_filter, d_bins);
  float tbl[256];
  filterTableHost(p.filter_kind, p.filter_params, P.fw, P.fh, tbl);
  RET_CUDA(cudaMemcpyAsync(d_filter, tbl, sizeof tbl, cudaMemcpyHostToDevice, stream));
  RET_CUDA(cudaMemsetAsync(counters, 0, C_COUNT * sizeof(unsigned long long), stream));
  int sms = 0;
  RET_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  Grids G = grids(device, sms);
  P.chunk_base = 0;
  RET_CUDA(runChunk(stream, A, S, P, st, Q, counters, (int64_t)total, p.max_depth, d_film, d_filter,
                    G, d_bins, nullptr));
  unsigned long long cnt[C_COUNT];
  RET_CUDA(cudaMemcpyAsync(cnt, counters, sizeof cnt, cudaMemcpyDeviceToHost, stream));
  RET_CUDA(cudaStreamSynchronize(stream));
  res.rays_closest = cnt[C_CLOSEST];
  res.rays_any = cnt[C_ANY];
  res.nonfinite = cnt[C_NONFINITE];
  res.degenerate = cnt[C_DEGENERATE];
  res.path_samples = total;
  firstDropped(P, cnt[C_FIRST_NONFINITE], res);
  return BLING_OK;
}

}  // namespace bgpu
