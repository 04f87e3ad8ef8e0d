// Batched job engine (batch.h): path regeneration over a table of jobs, one
// wavefront for all of them, each iteration's launches replayed from a CUDA
// graph.
//
// Path state lives in two buffers.  At the start of an iteration the paths
// of the current buffer sit at positions [0, n): the paths that continue from
// the previous iteration (compacted), then the paths started in this
// iteration, in sample order.  Every kernel indexes state by position, so
// the per-path loads and stores of trace, shade and resolve are coalesced;
// the resolve kernel writes each continuing path to the next free position
// of the other buffer.  Optional ray binning permutes the state into bin
// order through the other buffer before the traversal.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "batch.h"
#include "filter_host.h"
#include "wavefront.cuh"

namespace bgpu {

constexpr int kMaxBatchScenes = 1024;
constexpr int kBinBits = 16;
constexpr int kBins = 1 << kBinBits;

struct BatchSceneDev {
  DevAccel A;
  DevShading S;
  float lo[3], hi[3];  // world bounds (ray binning)
};

struct BatchJobDev {
  PassParams P;  // chunk_base unused: sample indices are job-relative
  bling_camera_desc cam;
  float* film;
  int32_t scene;
  int32_t pad;
  unsigned long long start, total;  // the job's samples in the engine's sample sequence
  unsigned long long offset;        // sample index (in the pass) of the job's first sample
  float filter[256];
};

// control block; the first four words are written by the host between steps
struct BatchCtl {
  unsigned long long end_sample;  // samples submitted
  unsigned long long job_lo;      // jobs [job_lo, job_hi) may still own samples (sequence numbers)
  unsigned long long job_hi;
  unsigned long long pad0;
  unsigned long long next_sample;  // the next sample to start
  unsigned long long regen_base, regen_count, regen_pos;
  unsigned long long finished;     // paths finished
  unsigned long long iterations;
  unsigned long long loop_iters;   // iterations in the current device-side loop
  unsigned long long pad1;
  unsigned long long c[C_COUNT];   // C_LIVE0 + b: paths in buffer b; queue sizes, statistics
  int cur;                         // the buffer traced this iteration
  int pad2;
  unsigned cls[32];                // shading-class counts [0, 16) and cursors [16, 32)
};

// the per-path state that moves between the two buffers
struct PathState {
  unsigned long long* gidx;  // job-relative sample index
  float* T;                  // 16 per path
  float* L;                  // 16 per path
  float* ray;                // 8 per path (sign of tmin: the previous bounce was specular)
  int32_t* job;              // job table index
  int32_t* scene;            // scene table index
  int32_t* depth;            // bounce of the path's current vertex
};
constexpr size_t kStateWords = 2 + 16 + 16 + 8 + 3;

struct PathStates {
  PathState b[2];
};

struct BatchQueues {
  int32_t* shadow;     // 2 cap entries: shadow rays and MIS rays (occlusionSlot)
  int32_t* resolve;
  uint32_t* keys;      // bin key per path
  int32_t* order;      // positions of the current buffer in shading-class order
  int32_t* cls;        // shading class per position
  unsigned int* bins;  // kBins counters / offsets
};
constexpr size_t kQueueWordsB = 6;  // the shadow queue takes two

// vertex temporaries (everything of Slots but T, L and ray), single-buffered
constexpr size_t kTempWords = kSlotWords - 16 - 16 - 8;

struct JobFilter {
  const float* t;
  __device__ __forceinline__ float operator()(int i) const { return __ldg(t + i); }
};

// Slots view of buffer b: its T, L and ray with the shared temporaries
__device__ __forceinline__ Slots viewOf(const Slots& tmp, const PathState& p) {
  Slots v = tmp;
  v.T = p.T;
  v.L = p.L;
  v.ray = p.ray;
  return v;
}

// warp-aggregated position in a queue (every lane of the warp calls it);
// -1 for lanes that do not append
__device__ __forceinline__ long long queueSlot(bool live, unsigned long long* count) {
  const unsigned mask = 0xffffffffu;
  __syncwarp();
  unsigned ballot = __ballot_sync(mask, live);
  if (!ballot) return -1;
  int lane = threadIdx.x & 31;
  int leader = __ffs(ballot) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(count, (unsigned long long)__popc(ballot));
  base = __shfl_sync(mask, base, leader);
  return live ? (long long)(base + __popc(ballot & ((1u << lane) - 1))) : -1;
}

__device__ __forceinline__ void moveState(const PathState& from, int q, const PathState& to,
                                          int p) {
  to.gidx[p] = from.gidx[q];
  storeBands(to.T, p, loadBands(from.T, q));
  storeBands(to.L, p, loadBands(from.L, q));
  copyRay(from.ray, q, to.ray, p);
  to.job[p] = from.job[q];
  to.scene[p] = from.scene[q];
  to.depth[p] = from.depth[q];
}

// ------------------------------------------------------------------ kernels
// hands the free positions of the current buffer to the next samples and
// resets the iteration's queue counters
__global__ void k_iter_begin(BatchCtl* ctl, unsigned long long cap) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int cur = ctl->cur;
  unsigned long long n_live = ctl->c[C_LIVE0 + cur];
  unsigned long long next = ctl->next_sample, end = ctl->end_sample;
  unsigned long long avail = end > next ? end - next : 0;
  unsigned long long room = cap > n_live ? cap - n_live : 0;
  unsigned long long nr = avail < room ? avail : room;
  ctl->regen_base = next;
  ctl->regen_count = nr;
  ctl->regen_pos = n_live;
  ctl->next_sample = next + nr;
  ctl->c[C_LIVE0 + cur] = n_live + nr;
  ctl->c[C_LIVE0 + 1 - cur] = 0;
  ctl->c[C_NEXT_TRACE] = 0;
  ctl->c[C_SHADOW] = 0;
  ctl->c[C_RESOLVE] = 0;
  ctl->c[C_NEXT_SHADOW] = 0;
  for (int k = 0; k < 32; k++) ctl->cls[k] = 0;
}

// the job owning sample g: the last of jobs [lo, hi) whose first sample is <= g
__device__ __forceinline__ int findJob(const BatchJobDev* __restrict__ jobs, unsigned mask,
                                       unsigned long long lo, unsigned long long hi,
                                       unsigned long long g) {
  while (hi - lo > 1) {
    unsigned long long mid = lo + (hi - lo) / 2;
    if (jobs[mid & mask].start <= g)
      lo = mid;
    else
      hi = mid;
  }
  return (int)(lo & mask);
}

// camera rays of the samples started this iteration (fireRay, Camera.hs:49-68)
__global__ void __launch_bounds__(128) k_regen(BatchCtl* ctl, const BatchJobDev* __restrict__ jobs,
                                               unsigned job_mask, PathStates ps, size_t cap) {
  const unsigned long long n = ctl->regen_count, base = ctl->regen_base;
  const unsigned long long lo = ctl->job_lo, hi = ctl->job_hi, pos = ctl->regen_pos;
  const PathState& S = ps.b[ctl->cur];
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    int q = (int)(pos + i);
    unsigned long long g = base + i;
    int j = findJob(jobs, job_mask, lo, hi, g);
    const BatchJobDev& J = jobs[j];
    unsigned long long local = g - J.start + J.offset;
    S.job[q] = j;
    S.scene[q] = J.scene;
    S.depth[q] = 0;
    S.gidx[q] = local;
    Ray ray = cameraRay(J.P, J.cam, local);
    storeRay(S.ray, q, ray);
    storeBands(S.T, q, sConst(1.0f));
    storeBands(S.L, q, sConst(0.0f));
  }
}

// ---- ray binning: a 16-bit key (6 bits of the scene index, the direction
// octant, the top 7 bits of the 9-bit Morton code of the origin's cell in an
// 8x8x8 grid over the scene's bounds), one counting pass, a scan, and a
// scatter that moves the path state into bin order in the other buffer.
// Order within a bin is arbitrary; it only changes which warp traces a ray.
__device__ __forceinline__ uint32_t spread3(uint32_t v) {  // 3 bits -> every third bit
  return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4);
}

__global__ void __launch_bounds__(128) k_bin_count(BatchCtl* ctl,
                                                   const BatchSceneDev* __restrict__ scenes,
                                                   PathStates ps, BatchQueues Q, size_t cap) {
  const int cur = ctl->cur;
  const unsigned long long n = ctl->c[C_LIVE0 + cur];
  const PathState& S = ps.b[cur];
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  const unsigned long long nround = (n + stride - 1) / stride * stride;
  const int lane = threadIdx.x & 31;
  for (unsigned long long q = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
       q < nround; q += stride) {
    uint32_t key = 0xffffffffu;
    if (q < n) {
      int sc = S.scene[q];
      const BatchSceneDev& B = scenes[sc];
      uint32_t cell = 0, oct = 0;
#pragma unroll
      for (int a = 0; a < 3; a++) {
        float o = S.ray[8 * (size_t)q + a], d = S.ray[8 * (size_t)q + 3 + a];
        float ext = B.hi[a] - B.lo[a];
        float u = ext > 0 ? (o - B.lo[a]) / ext : 0.0f;
        int v = (int)(u * 8.0f);
        v = v < 0 ? 0 : (v > 7 ? 7 : v);  // NaN -> 0
        cell |= spread3((uint32_t)v) << a;
        oct |= (signbit(d) ? 1u : 0u) << a;
      }
      key = ((uint32_t)(sc & 63) << 10) | (oct << 7) | (cell >> 2);
      Q.keys[q] = key;
    }
    // one atomic per distinct key in the warp
    unsigned grp = __match_any_sync(0xffffffffu, key);
    if (key != 0xffffffffu && lane == __ffs(grp) - 1) atomicAdd(Q.bins + key, (unsigned)__popc(grp));
  }
}

// exclusive scan of the kBins counters in place (one block)
__global__ void __launch_bounds__(1024) k_bin_scan(unsigned int* __restrict__ bins) {
  __shared__ unsigned int part[1024];
  constexpr int per = kBins / 1024;
  const int t = threadIdx.x;
  unsigned int sum = 0;
  for (int k = 0; k < per; k++) sum += bins[t * per + k];
  part[t] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    unsigned int v = t >= off ? part[t - off] : 0u;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  unsigned int run = part[t] - sum;
  for (int k = 0; k < per; k++) {
    unsigned int v = bins[t * per + k];
    bins[t * per + k] = run;
    run += v;
  }
}

__global__ void __launch_bounds__(128) k_bin_scatter(BatchCtl* ctl, PathStates ps, BatchQueues Q,
                                                     size_t cap) {
  const int cur = ctl->cur;
  const unsigned long long n = ctl->c[C_LIVE0 + cur];
  const PathState& from = ps.b[cur];
  const PathState& to = ps.b[1 - cur];
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  const unsigned long long nround = (n + stride - 1) / stride * stride;
  const int lane = threadIdx.x & 31;
  for (unsigned long long q = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
       q < nround; q += stride) {
    uint32_t key = q < n ? Q.keys[q] : 0xffffffffu;
    // one atomic per distinct key in the warp; lanes take consecutive positions
    unsigned grp = __match_any_sync(0xffffffffu, key);
    int leader = __ffs(grp) - 1;
    unsigned base = 0;
    if (key != 0xffffffffu && lane == leader) base = atomicAdd(Q.bins + key, (unsigned)__popc(grp));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (key != 0xffffffffu)
      moveState(from, (int)q, to, (int)(base + __popc(grp & ((1u << lane) - 1))));
  }
}

// the binned state becomes the current buffer
__global__ void k_bin_flip(BatchCtl* ctl) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int cur = ctl->cur;
  ctl->c[C_LIVE0 + 1 - cur] = ctl->c[C_LIVE0 + cur];
  ctl->c[C_LIVE0 + cur] = 0;
  ctl->cur = 1 - cur;
}

// closest hits of the current buffer's rays, each lane in its ray's scene
template <int LAYOUT>
__global__ void __launch_bounds__(128) k_btrace(BatchCtl* ctl,
                                                const BatchSceneDev* __restrict__ scenes,
                                                Slots tmp, PathStates ps) {
  const int cur = ctl->cur;
  const PathState& S = ps.b[cur];
  const size_t cap = tmp.cap;
  int64_t n = (int64_t)ctl->c[C_LIVE0 + cur];
  traceWarpPersistent<false, LAYOUT, false>(
      scenes[0].A, n, ctl->c + C_NEXT_TRACE,
      [&](int64_t q) { return loadRay7(S.ray, (int)q); },
      [&](int64_t q, const RayQueryResult& res) {
        tmp.hit[q] = hitRecord(res.hit, res.t, res.prim, res.b1, res.b2);
      },
      nullptr, [&](int64_t q) { return &scenes[S.scene[q]].A; });
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(ctl->c + C_CLOSEST, (unsigned long long)n);
}

template <int LAYOUT>
__global__ void __launch_bounds__(128) k_btrace_shadow(BatchCtl* ctl,
                                                       const BatchSceneDev* __restrict__ scenes,
                                                       Slots tmp, PathStates ps, BatchQueues Q) {
  const PathState& S = ps.b[ctl->cur];
  int64_t n = (int64_t)ctl->c[C_SHADOW];
  const int32_t* __restrict__ queue = Q.shadow;
  traceWarpPersistent<true, LAYOUT, false, true>(
      scenes[0].A, n, ctl->c + C_NEXT_SHADOW,
      [&](int64_t q, bool& by_intersect, int& rank_prim) {
        return loadOcclusionRay(tmp, queue[q], by_intersect, rank_prim);
      },
      [&](int64_t q, const RayQueryResult& res) {
        storeOcclusion(tmp, queue[q], res, ctl->c + C_DEGENERATE);
      },
      nullptr, [&](int64_t q) { return &scenes[S.scene[occlusionSlot(queue[q])]].A; });
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(ctl->c + C_ANY, (unsigned long long)n);
}


// Shading order of the current buffer: paths sorted by (job, shading class).
// Shading reads each path's job parameters and scene tables through the job
// and scene tables; grouping a job's paths keeps those loads uniform across a
// warp, and the class keeps its lanes on one BSDF's code.  The key is
// (job table index mod 4096) x 16 + class in the kBins counters: one
// counting pass, the scan of k_bin_scan, and a scatter of positions.  Order
// within a key is arbitrary; it only changes which warp shades a path.
__device__ __forceinline__ uint32_t shadeKey(int job, int cls) {
  return ((uint32_t)(job & 4095) << 4) | (uint32_t)cls;
}

__global__ void __launch_bounds__(128) k_bclass_count(BatchCtl* ctl,
                                                      const BatchSceneDev* __restrict__ scenes,
                                                      Slots tmp, PathStates ps, BatchQueues Q) {
  static_assert(kShadeClasses <= 16 && (4096u << 4) <= (unsigned)kBins, "shade keys fit the bins");
  const int cur = ctl->cur;
  const PathState& S = ps.b[cur];
  int64_t n = (int64_t)ctl->c[C_LIVE0 + cur];
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t nround = (n + stride - 1) / stride * stride;
  const int lane = threadIdx.x & 31;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nround; q += stride) {
    uint32_t key = 0xffffffffu;
    if (q < n) {
      const BatchSceneDev& SC = scenes[S.scene[q]];
      key = shadeKey(S.job[q], shadeClass(SC.A, SC.S, hitPrim(tmp.hit, q)));
      Q.keys[q] = key;
    }
    // one atomic per distinct key in the warp
    unsigned grp = __match_any_sync(0xffffffffu, key);
    if (key != 0xffffffffu && lane == __ffs(grp) - 1) atomicAdd(Q.bins + key, (unsigned)__popc(grp));
  }
}

// the positions of the current buffer in (job, class) order
__global__ void __launch_bounds__(128) k_bclass_scatter(BatchCtl* ctl, BatchQueues Q) {
  int64_t n = (int64_t)ctl->c[C_LIVE0 + ctl->cur];
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t nround = (n + stride - 1) / stride * stride;
  const int lane = threadIdx.x & 31;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nround; q += stride) {
    uint32_t key = q < n ? Q.keys[q] : 0xffffffffu;
    unsigned grp = __match_any_sync(0xffffffffu, key);
    int leader = __ffs(grp) - 1;
    unsigned base = 0;
    if (key != 0xffffffffu && lane == leader) base = atomicAdd(Q.bins + key, (unsigned)__popc(grp));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (key != 0xffffffffu) Q.order[base + __popc(grp & ((1u << lane) - 1))] = (int32_t)q;
  }
}

// a warp's finished paths: their jobs' sample counts go up (one atomic per
// job present in the warp)
__device__ __forceinline__ void pathsDone(bool fin, int job, BatchCtl* ctl,
                                          unsigned long long* __restrict__ job_done) {
  const unsigned FULL = 0xffffffffu;
  unsigned grp = __match_any_sync(FULL, fin ? job : -1);
  int lane = threadIdx.x & 31;
  if (fin && lane == __ffs(grp) - 1) atomicAdd(job_done + job, (unsigned long long)__popc(grp));
  unsigned b = __ballot_sync(FULL, fin);
  if (b && lane == 0) atomicAdd(&ctl->finished, (unsigned long long)__popc(b));
}

// TEX: some registered scene has textured materials
template <bool TEX>
__global__ void __launch_bounds__(128, 3) k_bshade(BatchCtl* ctl, const BatchJobDev* __restrict__ jobs,
                                                const BatchSceneDev* __restrict__ scenes,
                                                Slots tmp, PathStates ps, BatchQueues Q,
                                                unsigned long long* __restrict__ job_done) {
  const int cur = ctl->cur;
  const PathState& S = ps.b[cur];
  const Slots st = viewOf(tmp, S);
  unsigned long long* c = ctl->c;
  int64_t n = (int64_t)c[C_LIVE0 + cur];
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t nround = (n + stride - 1) / stride * stride;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nround; i += stride) {
    VertexOut o{false, false, false};
    bool fin = false;
    int job = -1;
    int q = 0;
    if (i < n) {
      q = Q.order[i];  // shading-class order
      job = S.job[q];
      const BatchJobDev& J = jobs[job];
      const BatchSceneDev& SC = scenes[S.scene[q]];
      unsigned long long g = S.gidx[q];
      o = shadeVertex<TEX>(SC.A, SC.S, J.P, st, (int)q, g, S.depth[q], c, [&](const Spec& L) {
        splatSample(J.film, J.P, g, L, c, JobFilter{J.filter});
        fin = true;
      });
    }
    queueAppend(o.shadow, (int)q, Q.shadow, c + C_SHADOW);
    queueAppend(o.mis, ~(int)q, Q.shadow, c + C_SHADOW);
    queueAppend(o.resolve, (int)q, Q.resolve, c + C_RESOLVE);
    pathsDone(fin, job, ctl, job_done);
  }
}

// the vertex's radiance; continuing paths move to the next free position of
// the other buffer, finished ones are splatted into their job's film
__global__ void __launch_bounds__(128, 3) k_bresolve(BatchCtl* ctl,
                                                  const BatchJobDev* __restrict__ jobs,
                                                  const BatchSceneDev* __restrict__ scenes,
                                                  Slots tmp, PathStates ps, BatchQueues Q,
                                                  unsigned long long* __restrict__ job_done) {
  const int cur = ctl->cur, nxt = 1 - cur;
  const PathState& S = ps.b[cur];
  const PathState& D = ps.b[nxt];
  const Slots st = viewOf(tmp, S);
  const size_t cap = tmp.cap;
  unsigned long long* c = ctl->c;
  int64_t n = (int64_t)c[C_RESOLVE];
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t nround = (n + stride - 1) / stride * stride;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nround; i += stride) {
    bool cont = false, fin = false;
    int q = 0, job = -1;
    Spec Tn, Ln;
    if (i < n) {
      q = Q.resolve[i];
      job = S.job[q];
      const BatchJobDev& J = jobs[job];
      const BatchSceneDev& SC = scenes[S.scene[q]];
      unsigned long long g = S.gidx[q];
      cont = resolveVertex(
          SC.A, SC.S, st, q, c,
          [&](const Spec& L) {
            splatSample(J.film, J.P, g, L, c, JobFilter{J.filter});
            fin = true;
          },
          Tn, Ln);
    }
    long long p = queueSlot(cont, c + C_LIVE0 + nxt);
    if (cont) {
      storeBands(D.T, (int)p, Tn);
      storeBands(D.L, (int)p, Ln);
      copyRay(S.ray, q, D.ray, (int)p);
      D.gidx[p] = S.gidx[q];
      D.job[p] = job;
      D.scene[p] = S.scene[q];
      D.depth[p] = S.depth[q] + 1;
    }
    pathsDone(fin, job, ctl, job_done);
  }
}

// flips the buffers; in the device-side loop also decides whether the loop
// runs another iteration (work left and the launch's budget not spent)
__global__ void k_iter_end(BatchCtl* ctl, cudaGraphConditionalHandle handle, int use_cond,
                           unsigned long long max_iters) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  ctl->cur ^= 1;
  ctl->iterations += 1;
  if (use_cond) {
    unsigned long long li = ++ctl->loop_iters;
    bool work = ctl->c[C_LIVE0 + ctl->cur] > 0 || ctl->next_sample < ctl->end_sample;
    cudaGraphSetConditional(handle, (work && li < max_iters) ? 1u : 0u);
  }
}

// drops the paths in flight and stops sample generation at `end` (batch_cancel)
__global__ void k_cancel(BatchCtl* ctl, unsigned long long end) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  ctl->next_sample = end;
  ctl->regen_count = 0;
  ctl->c[C_LIVE0] = 0;
  ctl->c[C_LIVE0 + 1] = 0;
}

// ------------------------------------------------------------------ host side
struct BatchEngine {
  int device = 0;
  cudaStream_t stream = nullptr;
  BatchConfig cfg;
  int64_t cap = 0;
  unsigned job_mask = 0;
  void* buf = nullptr;  // path states, temporaries, queues, bins
  size_t buf_bytes = 0;
  BatchCtl* d_ctl = nullptr;
  BatchJobDev* d_jobs = nullptr;
  unsigned long long* d_job_done = nullptr;
  BatchSceneDev* d_scenes = nullptr;
  Slots tmp{};
  PathStates ps{};
  BatchQueues q{};
  std::vector<uint64_t> scene_keys;  // scene serial numbers, by table index
  int wide = -1;  // node layout of the registered scenes
  bool textured = false;  // some registered scene has textured materials
  // host mirror of the job table
  unsigned long long end_sample = 0, job_lo = 0, job_hi = 0;
  struct JobHost {
    unsigned long long total = 0, done = 0;
  };
  std::vector<JobHost> jobs;
  std::vector<unsigned long long> done_buf;
  std::vector<unsigned long long> totals;  // sample count of every job ever submitted
  bool ctl_dirty = true;
  // launch shapes
  unsigned g_trace = 0, g_shadow = 0, g_shade = 0, g_resolve = 0, g_regen = 0,
           g_bin = 0;
  // graphs
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphConditionalHandle cond = 0;
  BatchStats stats;
};

namespace {

#define BRET(call)                                                                   \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);                      \
      return e_ == cudaErrorMemoryAllocation ? BLING_ERR_OOM : BLING_ERR_CUDA;       \
    }                                                                                \
  } while (0)

template <class K>
unsigned residentBlocks(K kernel, int block, int sms) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
  return (unsigned)(std::max(1, sms) * std::max(1, per_sm));
}

template <int LAYOUT>
void shapesFor(BatchEngine* b, int sms) {
  const int bl = b->cfg.block;
  b->g_trace = residentBlocks(k_btrace<LAYOUT>, bl, sms);
  b->g_shadow = residentBlocks(k_btrace_shadow<LAYOUT>, bl, sms);
}

// one iteration's launches, in order, on b->stream
template <int LAYOUT>
cudaError_t enqueueIterationT(BatchEngine* b, int use_cond, unsigned long long max_iters) {
  const int bl = b->cfg.block;
  const size_t cap = (size_t)b->cap;
  cudaStream_t s = b->stream;
  k_iter_begin<<<1, 32, 0, s>>>(b->d_ctl, (unsigned long long)cap);
  k_regen<<<b->g_regen, bl, 0, s>>>(b->d_ctl, b->d_jobs, b->job_mask, b->ps, cap);
  if (b->cfg.sort_rays) {
    cudaMemsetAsync(b->q.bins, 0, sizeof(unsigned int) * kBins, s);
    k_bin_count<<<b->g_bin, 128, 0, s>>>(b->d_ctl, b->d_scenes, b->ps, b->q, cap);
    k_bin_scan<<<1, 1024, 0, s>>>(b->q.bins);
    k_bin_scatter<<<b->g_bin, 128, 0, s>>>(b->d_ctl, b->ps, b->q, cap);
    k_bin_flip<<<1, 32, 0, s>>>(b->d_ctl);
  }
  k_btrace<LAYOUT><<<b->g_trace, bl, 0, s>>>(b->d_ctl, b->d_scenes, b->tmp, b->ps);
  cudaMemsetAsync(b->q.bins, 0, sizeof(unsigned int) * kBins, s);
  k_bclass_count<<<b->g_bin, 128, 0, s>>>(b->d_ctl, b->d_scenes, b->tmp, b->ps, b->q);
  k_bin_scan<<<1, 1024, 0, s>>>(b->q.bins);
  k_bclass_scatter<<<b->g_bin, 128, 0, s>>>(b->d_ctl, b->q);
  if (b->textured)
    k_bshade<true><<<b->g_shade, bl, 0, s>>>(b->d_ctl, b->d_jobs, b->d_scenes, b->tmp, b->ps,
                                             b->q, b->d_job_done);
  else
    k_bshade<false><<<b->g_shade, bl, 0, s>>>(b->d_ctl, b->d_jobs, b->d_scenes, b->tmp, b->ps,
                                              b->q, b->d_job_done);
  k_btrace_shadow<LAYOUT><<<b->g_shadow, bl, 0, s>>>(b->d_ctl, b->d_scenes, b->tmp, b->ps, b->q);
  k_bresolve<<<b->g_resolve, bl, 0, s>>>(b->d_ctl, b->d_jobs, b->d_scenes, b->tmp, b->ps, b->q,
                                         b->d_job_done);
  k_iter_end<<<1, 32, 0, s>>>(b->d_ctl, b->cond, use_cond, max_iters);
  return cudaGetLastError();
}

cudaError_t enqueueIteration(BatchEngine* b, int use_cond, unsigned long long max_iters) {
  return withLayout(b->wide, [&](auto L) {
    return enqueueIterationT<decltype(L)::value>(b, use_cond, max_iters);
  });
}

int launchShapes(BatchEngine* b, std::string& err) {
  int sms = 0;
  BRET(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device));
  const int bl = b->cfg.block;
  withLayout(b->wide, [&](auto L) { shapesFor<decltype(L)::value>(b, sms); });
  unsigned cap_blocks = (unsigned)std::max<int64_t>(1, (b->cap + bl - 1) / bl);
  b->g_shade = std::min(residentBlocks(k_bshade<false>, bl, sms), cap_blocks);
  b->g_resolve = std::min(residentBlocks(k_bresolve, bl, sms), cap_blocks);
  b->g_regen = std::min(residentBlocks(k_regen, bl, sms), cap_blocks);
  b->g_bin = std::min<unsigned>((unsigned)sms * 16u,
                                (unsigned)std::max<int64_t>(1, (b->cap + 127) / 128));
  b->g_trace = std::min(b->g_trace, cap_blocks);
  b->g_shadow = std::min(b->g_shadow, cap_blocks);
  return BLING_OK;
}

int buildGraph(BatchEngine* b, std::string& err) {
  if (b->exec || (b->cfg.graph_mode == 0 && b->g_trace)) return BLING_OK;
  int rc = launchShapes(b, err);
  if (rc) return rc;
  if (b->cfg.graph_mode == 0) return BLING_OK;
  cudaStreamCaptureStatus cs;
  BRET(cudaStreamIsCapturing(b->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) {
    err = "the batch's stream is being captured by the caller";
    return BLING_ERR_STATE;
  }
  BRET(cudaGraphCreate(&b->graph, 0));
  if (b->cfg.graph_mode == 1) {
    BRET(cudaStreamBeginCaptureToGraph(b->stream, b->graph, nullptr, nullptr, 0,
                                       cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueueIteration(b, 0, 0);
    cudaGraph_t out = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &out);
    BRET(e);
    BRET(e2);
  } else {
    // a while node whose body is one iteration; k_iter_end sets its condition
    BRET(cudaGraphConditionalHandleCreate(&b->cond, b->graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = b->cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    BRET(cudaGraphAddNode(&node, b->graph, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    BRET(cudaStreamBeginCaptureToGraph(b->stream, body, nullptr, nullptr, 0,
                                       cudaStreamCaptureModeThreadLocal));
    cudaError_t e =
        enqueueIteration(b, 1, (unsigned long long)std::max(1, b->cfg.iters_per_launch));
    cudaGraph_t out = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &out);
    BRET(e);
    BRET(e2);
  }
  BRET(cudaGraphInstantiate(&b->exec, b->graph, 0));
  return BLING_OK;
}

int syncHostCtl(BatchEngine* b, std::string& err) {
  if (!b->ctl_dirty) return BLING_OK;
  unsigned long long h[4] = {b->end_sample, b->job_lo, b->job_hi, 0};
  BRET(cudaMemcpyAsync(b->d_ctl, h, sizeof h, cudaMemcpyHostToDevice, b->stream));
  b->ctl_dirty = false;
  return BLING_OK;
}

}  // namespace

int batch_create(int device, cudaStream_t stream, const BatchConfig& cfg, BatchEngine** out,
                 std::string& err) {
  *out = nullptr;
  if (cfg.slots < 1024 || cfg.slots > (int64_t(1) << 27)) {
    err = "batch slots must be in [1024, 2^27]";
    return BLING_ERR_INVALID_ARG;
  }
  static_assert(128 <= kMaxTraceBlock, "batch blocks must fit the traversal's shared stack");
  if (cfg.block != 64 && cfg.block != 128) {
    err = "batch block size must be 64 or 128";
    return BLING_ERR_INVALID_ARG;
  }
  if (cfg.max_jobs < 1 || cfg.max_jobs > (1 << 20) || (cfg.max_jobs & (cfg.max_jobs - 1))) {
    err = "batch max_jobs must be a power of two in [1, 2^20]";
    return BLING_ERR_INVALID_ARG;
  }
  if (cfg.graph_mode < 0 || cfg.graph_mode > 2 || cfg.iters_per_launch < 1) {
    err = "batch graph_mode must be 0, 1 or 2 and iters_per_launch >= 1";
    return BLING_ERR_INVALID_ARG;
  }
  std::unique_ptr<BatchEngine> b(new BatchEngine());
  b->device = device;
  b->stream = stream;
  b->cfg = cfg;
  // a multiple of 64 paths keeps every per-path array 16-byte aligned (the
  // records are read with 16-byte vector loads)
  b->cap = (cfg.slots + 63) / 64 * 64;
  b->job_mask = (unsigned)cfg.max_jobs - 1;
  b->jobs.resize(cfg.max_jobs);
  b->done_buf.resize(cfg.max_jobs);
  BRET(loadCieConstants(device));
  const size_t cap = (size_t)b->cap;
  // two path states, the vertex temporaries, the queues, the bin counters
  size_t words = (2 * kStateWords + kTempWords + kQueueWordsB) * cap;
  b->buf_bytes = words * 4 + sizeof(unsigned int) * kBins + 256;
  BRET(cudaMalloc(&b->buf, b->buf_bytes));
  float* w = (float*)b->buf;
  auto take = [&](size_t n) {
    float* p = w;
    w += n * cap;
    return p;
  };
  for (int k = 0; k < 2; k++) {  // the 8-byte arrays first: every offset is a multiple of 8 bytes
    b->ps.b[k].gidx = (unsigned long long*)take(2);
  }
  for (int k = 0; k < 2; k++) {
    PathState& p = b->ps.b[k];
    p.T = take(16);
    p.L = take(16);
    p.ray = take(8);
    p.job = (int32_t*)take(1);
    p.scene = (int32_t*)take(1);
    p.depth = (int32_t*)take(1);
  }
  Slots& t = b->tmp;
  t.cap = cap;
  t.T = t.L = t.ray = nullptr;  // per buffer (viewOf)
  t.hit = reinterpret_cast<float4*>(take(4));
  t.intl = take(16);
  t.ls = take(16);
  t.bsf = take(16);
  t.fc = take(16);
  t.bsw = take(1);
  t.invpc = take(1);
  t.vflags = (int32_t*)take(1);
  t.sray = take(8);
  t.svis = (int32_t*)take(1);
  t.mray = take(8);
  t.mhit = reinterpret_cast<float4*>(take(4));
  b->q.shadow = (int32_t*)take(2);  // shadow rays and MIS rays
  b->q.resolve = (int32_t*)take(1);
  b->q.keys = (uint32_t*)take(1);
  b->q.order = (int32_t*)take(1);
  b->q.cls = (int32_t*)take(1);
  b->q.bins = (unsigned int*)w;
  BRET(cudaMalloc(&b->d_ctl, sizeof(BatchCtl)));
  BRET(cudaMalloc(&b->d_jobs, sizeof(BatchJobDev) * cfg.max_jobs));
  BRET(cudaMalloc(&b->d_job_done, sizeof(unsigned long long) * cfg.max_jobs));
  BRET(cudaMalloc(&b->d_scenes, sizeof(BatchSceneDev) * kMaxBatchScenes));
  BRET(cudaMemsetAsync(b->d_ctl, 0, sizeof(BatchCtl), stream));
  BRET(cudaMemsetAsync(b->d_job_done, 0, sizeof(unsigned long long) * cfg.max_jobs, stream));
  BRET(cudaStreamSynchronize(stream));
  b->stats.device_bytes = (double)(b->buf_bytes + sizeof(BatchCtl) +
                                   (sizeof(BatchJobDev) + 8) * cfg.max_jobs +
                                   sizeof(BatchSceneDev) * kMaxBatchScenes);
  *out = b.release();
  return BLING_OK;
}

void batch_destroy(BatchEngine* b) {
  if (!b) return;
  cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  cudaFree(b->buf);
  cudaFree(b->d_ctl);
  cudaFree(b->d_jobs);
  cudaFree(b->d_job_done);
  cudaFree(b->d_scenes);
  delete b;
}

bool batch_uses_wide(BatchEngine* b) { return b && b->wide == 1; }

int batch_scene(BatchEngine* b, uint64_t key, const DevAccel& A, const DevShading& S,
                const float lo[3], const float hi[3], int& index, std::string& err) {
  for (size_t i = 0; i < b->scene_keys.size(); i++)
    if (b->scene_keys[i] == key) {
      index = (int)i;
      return BLING_OK;
    }
  if ((int)b->scene_keys.size() >= kMaxBatchScenes) {
    err = "batch scene table full";
    return BLING_ERR_BOUNDS;
  }
  int wide = A.wide;
  if (b->wide >= 0 && b->wide != wide) {
    err = "all scenes of a batch must use the same BVH layout";
    return BLING_ERR_INVALID_ARG;
  }
  b->wide = wide;
  if (S.textured && !b->textured) {
    // the iteration graph was captured with the untextured shading kernel
    b->textured = true;
    if (b->exec) {
      BRET(cudaStreamSynchronize(b->stream));
      cudaGraphExecDestroy(b->exec);
      b->exec = nullptr;
    }
    if (b->graph) {
      cudaGraphDestroy(b->graph);
      b->graph = nullptr;
    }
  }
  BatchSceneDev h;
  memset(&h, 0, sizeof h);
  h.A = A;
  h.S = S;
  for (int a = 0; a < 3; a++) {
    h.lo[a] = lo[a];
    h.hi[a] = hi[a];
  }
  index = (int)b->scene_keys.size();
  BRET(cudaMemcpyAsync(b->d_scenes + index, &h, sizeof h, cudaMemcpyHostToDevice, b->stream));
  BRET(cudaStreamSynchronize(b->stream));
  b->scene_keys.push_back(key);
  return BLING_OK;
}

int batch_submit(BatchEngine* b, int scene, const bling_camera_desc& cam, float* d_film, int fw,
                 int fh, const bling_render_params& p, uint64_t pass, int64_t& job_id,
                 std::string& err, uint64_t first, uint64_t count) {
  if (scene < 0 || scene >= (int)b->scene_keys.size()) {
    err = "unknown batch scene";
    return BLING_ERR_INVALID_ARG;
  }
  if (b->job_hi - b->job_lo >= (unsigned long long)b->cfg.max_jobs) {
    err = "batch job table full: step the batch until jobs complete";
    return BLING_ERR_STATE;
  }
  BatchJobDev h;
  memset(&h, 0, sizeof h);
  int rc = integrator_pass_params(p, pass, fw, fh, h.P, err);
  if (rc) return rc;
  uint64_t total = (uint64_t)h.P.nx * h.P.ny * h.P.spp;
  if (total == 0 || total >= (uint64_t(1) << 40)) {
    err = "job sample count out of range";
    return BLING_ERR_INVALID_ARG;
  }
  // a slice [first, first + count) of the pass's samples (count 0: the rest)
  if (first >= total || count > total - first) {
    err = "sample range outside the pass";
    return BLING_ERR_INVALID_ARG;
  }
  if (count == 0) count = total - first;
  h.offset = first;
  total = count;
  filterTableHost(p.filter_kind, p.filter_params, h.P.fw, h.P.fh, h.filter);
  h.cam = cam;
  h.film = d_film;
  h.scene = scene;
  h.start = b->end_sample;
  h.total = total;
  unsigned long long seq = b->job_hi;
  unsigned idx = (unsigned)(seq & b->job_mask);
  BRET(cudaMemcpyAsync(b->d_jobs + idx, &h, sizeof h, cudaMemcpyHostToDevice, b->stream));
  BRET(cudaMemsetAsync(b->d_job_done + idx, 0, sizeof(unsigned long long), b->stream));
  b->jobs[idx].total = total;
  b->jobs[idx].done = 0;
  b->totals.push_back(total);
  b->end_sample += total;
  b->job_hi = seq + 1;
  b->ctl_dirty = true;
  b->stats.jobs_submitted += 1;
  b->stats.samples_submitted += total;
  job_id = (int64_t)seq;
  return BLING_OK;
}

int batch_step(BatchEngine* b, int iterations, std::string& err) {
  if (iterations < 1) {
    err = "iterations must be >= 1";
    return BLING_ERR_INVALID_ARG;
  }
  if (b->job_lo == b->job_hi) return BLING_OK;  // nothing to do
  int rc = buildGraph(b, err);
  if (rc) return rc;
  rc = syncHostCtl(b, err);
  if (rc) return rc;
  if (b->cfg.graph_mode == 0) {
    for (int i = 0; i < iterations; i++) BRET(enqueueIteration(b, 0, 0));
  } else if (b->cfg.graph_mode == 1) {
    for (int i = 0; i < iterations; i++) BRET(cudaGraphLaunch(b->exec, b->stream));
  } else {
    int per = std::max(1, b->cfg.iters_per_launch);
    for (int done = 0; done < iterations; done += per) {
      BRET(cudaMemsetAsync(&b->d_ctl->loop_iters, 0, sizeof(unsigned long long), b->stream));
      BRET(cudaGraphLaunch(b->exec, b->stream));
    }
  }
  BatchCtl ctl;
  BRET(cudaMemcpyAsync(&ctl, b->d_ctl, sizeof ctl, cudaMemcpyDeviceToHost, b->stream));
  BRET(cudaMemcpyAsync(b->done_buf.data(), b->d_job_done,
                       sizeof(unsigned long long) * b->done_buf.size(), cudaMemcpyDeviceToHost,
                       b->stream));
  BRET(cudaStreamSynchronize(b->stream));
  for (unsigned long long s = b->job_lo; s < b->job_hi; s++) {
    auto& j = b->jobs[s & b->job_mask];
    j.done = b->done_buf[s & b->job_mask];
  }
  unsigned long long lo = b->job_lo;
  while (lo < b->job_hi && b->jobs[lo & b->job_mask].done >= b->jobs[lo & b->job_mask].total) lo++;
  if (lo != b->job_lo) {
    b->stats.jobs_done += (int64_t)(lo - b->job_lo);
    b->job_lo = lo;
    b->ctl_dirty = true;
  }
  b->stats.rays_closest = ctl.c[C_CLOSEST];
  b->stats.rays_any = ctl.c[C_ANY];
  b->stats.nonfinite = ctl.c[C_NONFINITE];
  b->stats.degenerate = ctl.c[C_DEGENERATE];
  b->stats.path_samples = ctl.finished;
  b->stats.iterations = ctl.iterations;
  b->stats.samples_started = ctl.next_sample;
  b->stats.jobs_active = (int64_t)(b->job_hi - b->job_lo);
  return BLING_OK;
}

int batch_run(BatchEngine* b, std::string& err) {
  // an iteration advances every live path by one bounce, so no job needs more
  // than (samples / slots + 1) * (max depth + 1) iterations; the bound keeps a
  // logic error from looping forever
  const int per = b->cfg.graph_mode == 2 ? std::max(1, b->cfg.iters_per_launch) * 4 : 8;
  const unsigned long long limit =
      b->cfg.max_run_iterations > 0
          ? (unsigned long long)b->cfg.max_run_iterations
          : ((b->end_sample / (unsigned long long)b->cap) + 2) * 4096ull + 1000000ull;
  unsigned long long spent = 0;
  while (b->job_lo < b->job_hi) {
    if (spent >= limit) {
      char buf[128];
      snprintf(buf, sizeof buf, "batch did not finish within its bound of %llu iterations",
               limit);
      err = buf;
      return BLING_ERR_TIMEOUT;
    }
    int n = (int)std::min<unsigned long long>((unsigned long long)per, limit - spent);
    int rc = batch_step(b, n, err);
    if (rc) return rc;
    spent += (unsigned long long)n;
  }
  return BLING_OK;
}

int batch_cancel(BatchEngine* b, std::string& err) {
  BRET(cudaStreamSynchronize(b->stream));
  k_cancel<<<1, 32, 0, b->stream>>>(b->d_ctl, b->end_sample);
  BRET(cudaGetLastError());
  if (b->job_lo != b->job_hi) {
    b->stats.jobs_done += (int64_t)(b->job_hi - b->job_lo);
    b->job_lo = b->job_hi;
  }
  b->ctl_dirty = true;
  int rc = syncHostCtl(b, err);
  if (rc) return rc;
  BRET(cudaStreamSynchronize(b->stream));
  b->stats.samples_started = b->end_sample;
  b->stats.jobs_active = 0;
  return BLING_OK;
}

int batch_job_status(BatchEngine* b, int64_t job_id, uint64_t& done, uint64_t& total,
                     std::string& err) {
  if (job_id < 0 || (unsigned long long)job_id >= b->job_hi) {
    err = "unknown job id";
    return BLING_ERR_INVALID_ARG;
  }
  if ((unsigned long long)job_id < b->job_lo) {
    // retired: complete (its table entry may have been reused)
    done = total = b->totals[(size_t)job_id];
    return BLING_OK;
  }
  const auto& j = b->jobs[(unsigned long long)job_id & b->job_mask];
  done = j.done;
  total = j.total;
  return BLING_OK;
}

void batch_stats(BatchEngine* b, BatchStats& out) { out = b->stats; }

}  // namespace bgpu
