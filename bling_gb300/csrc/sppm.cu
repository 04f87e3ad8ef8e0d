// Stochastic progressive photon mapping on the GPU.
//
// One pass of the reference's SPPM renderer (Renderer/SPPM.hs:410-480):
//
// 1. Camera pass (mkHitPoints, traceCam/followCam, SPPM.hs:77-164): one
//    Random-sampler camera sample per pixel of the sample extent.  At every
//    hit the path records a hit point if the BSDF has a non-specular part,
//    then follows BOTH its specular reflection and its specular transmission
//    (sampleBsdf' [prop, Specular]); emission seen along the way, and the
//    environment of escaping rays, goes to the film as a camera sample
//    (addSample).  The branching paths are a wavefront of nodes, each with
//    its sample and its position in the sample's binary tree (heap index);
//    the tree position keys the node's random numbers.
// 2. Spatial hash (mkHash, SPPM.hs:297-353): cells of twice the largest
//    radius over the hit points' bounds, one bucket per hit point, every hit
//    point entered in the buckets of the cells its sphere's box covers, with
//    the reference's cell hash.  A bucket is scanned linearly instead of
//    through the reference's per-bucket kd-tree: both visit the bucket's hit
//    points within their radius.
// 3. Photon pass (tracePhoton/followPhoton, SPPM.hs:170-243): ceil(sqrt n)^2
//    photons with stratified sampler dimensions; at every non-specular hit the
//    hit points of the hit's bucket within their radius get
//    hpF * f * li / (|wi.ng| r^2 pi) splatted at their pixel and a photon
//    counted; the photon continues by adjoint BSDF sampling, with Russian
//    roulette (0.8) after its eighth vertex.
// 4. Radius update (statsUpdate, SPPM.hs:272-295).
//
// The reference seeds its generators from system entropy; here the camera
// pass keys the shared counter-based generator by (seed, 2 pass, pixel) and
// the photon pass by (seed, 2 pass + 1, photon).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "filter_host.h"
#include "photon.cuh"
#include "sppm.h"

namespace bgpu {

namespace {

enum : int {
  S_NODES0 = 0, S_NODES1 = 1, S_NEXT_TRACE = 2, S_CLOSEST = 3, S_HP = 4, S_NODE_OVF = 5,
  S_NONFINITE = 6, S_DEGENERATE = 7, S_PLIVE0 = 8, S_PLIVE1 = 9, S_SPLATS = 10,
  // S_CLOSEST, S_NONFINITE, S_DEGENERATE as they were before the camera chunk
  // being run, restored when the chunk runs again with larger buffers
  S_SAVED_CLOSEST = 11, S_SAVED_NONFINITE = 12, S_SAVED_DEGENERATE = 13,
  S_COUNT = 16
};
// 32-bit words after the 8-byte counters: r2 max (float bits), ordered p min/max
constexpr int kBoundsAt = S_COUNT * 2;
constexpr size_t kSpCounterBytes = 256;

// the camera tree's random dimensions: 3 per node, by heap index
constexpr uint32_t kDimCamTree = 3u << 20;

struct CamNodes {
  float* ray;   // 8 per node
  float* T;     // 16 per node: throughput
  int2* id;     // (sample, heap index)
  float4* hit;
};
struct SpCam {
  float* Ls;  // 16 per sample: emission gathered by the sample's tree
  CamNodes nb[2];
  size_t C, NC;
};
struct SpHp {
  float4* p;    // shading point, radius^2
  float4* pix;  // raster position x, y, material (int bits)
  float4* w;    // wo
  float4* ng;   // geometric normal
  float4* sn;   // shading normal
  float4* sd;   // shading dpdu
  float* F;     // 16 per hit point: throughput
  size_t H;
};
struct SpHash {
  V3 lo;
  float scale;       // 1 / cell size
  long long cnt;     // buckets
  const uint32_t* off;  // cnt + 1 offsets into entries
  const int32_t* entries;  // hit-point index per entry
  const float4* epos;      // the entry's hit point: position, radius^2 (a copy, read in bucket order)
};
struct SpPhotons {
  float* li[2];   // 16 per photon: the power at this vertex / at the next (by depth parity)
  float* ray;
  float4* hit;
  float4* gpos;   // this vertex's hit: position, bucket (int bits; -1: no lookup)
  float4* gwi;    // this vertex's wi, |wi . ng|
  int32_t* live[2];
};
struct PhotonParams {
  uint64_t seed, pass;  // the photon pass's sampler key: (seed, 2 pass + 1, pixel 0 0)
  uint64_t chunk_base;
  int sn;
  V3 wc;
  float wr;
};

// sIdx (SPPM.hs:264-274): a raster position's entry in the pixel statistics
__device__ __forceinline__ int64_t statIndex(const PassParams& P, float px, float py) {
  int w = P.x1 - P.x0, h = P.y1 - P.y0;
  int ix = min(w, (int)px), iy = min(h, (int)py);  // truncate
  return (int64_t)w * (iy - P.y0) + (ix - P.x0);
}

// hash (SPPM.hs:303-305) and the bucket of a cell
__host__ __device__ __forceinline__ long long cellBucket(long long x, long long y, long long z,
                                                         long long cnt) {
  long long h = (long long)((unsigned long long)x * 73856093ull ^ (unsigned long long)y * 19349663ull ^
                            (unsigned long long)z * 83492791ull);
  h = h < 0 ? -h : h;
  long long r = h % cnt;
  return r < 0 ? 0 : (r > cnt - 1 ? cnt - 1 : r);
}

// warp-aggregated append: the position of this lane's entry, -1 if none
__device__ __forceinline__ long long appendPos(bool want, unsigned long long* count) {
  const unsigned mask = 0xffffffffu;
  unsigned ballot = __ballot_sync(mask, want);
  if (!ballot) return -1;
  int lane = threadIdx.x & 31;
  int leader = __ffs(ballot) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(count, (unsigned long long)__popc(ballot));
  base = __shfl_sync(mask, base, leader);
  return want ? (long long)(base + __popc(ballot & ((1u << lane) - 1))) : -1;
}

__device__ __forceinline__ void atomicAddBands(float* base, int s, const Spec& v) {
  float* p = base + 16 * (size_t)s;
#pragma unroll
  for (int i = 0; i < 16; i++) atomicAdd(p + i, v.v[i]);
}

__device__ __forceinline__ uint32_t orderedBits(float f) {
  uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
inline float fromOrdered(uint32_t o) {
  uint32_t b = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
  float f;
  memcpy(&f, &b, 4);
  return f;
}

// ------------------------------------------------------------------ camera pass
__global__ void __launch_bounds__(128) k_sp_camgen(PassParams P, bling_camera_desc cam, SpCam cs,
                                                   int64_t count, unsigned long long* counters) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    Ray ray = cameraRay(P, cam, P.chunk_base + (uint64_t)i);
    storeRay(cs.nb[0].ray, (int)i, ray);
    storeBands(cs.nb[0].T, (int)i, sConst(1.0f));
    cs.nb[0].id[i] = make_int2((int)i, 1);
    storeBands(cs.Ls, (int)i, sConst(0.0f));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) counters[S_NODES0] = (unsigned long long)count;
}

__global__ void k_sp_reset(unsigned long long* counters, int next) {
  if (threadIdx.x == 0) counters[next] = 0;
  if (threadIdx.x == 1) counters[S_NEXT_TRACE] = 0;
}

// a queue's node count: appends past the capacity were dropped (and counted
// as an overflow, after which the chunk runs again)
__device__ __forceinline__ int64_t nodeCount(const unsigned long long* counters, int q, size_t cap) {
  return (int64_t)min(counters[S_NODES0 + q], (unsigned long long)cap);
}

template <int LAYOUT>
__global__ void __launch_bounds__(128, 8) k_sp_camtrace(DevAccel A, CamNodes nb, int in, size_t cap,
                                                         unsigned long long* __restrict__ counters) {
  int64_t n = nodeCount(counters, in, cap);
  traceWarpPersistent<false, LAYOUT, false>(
      A, n, counters + S_NEXT_TRACE, [&](int64_t q) { return loadRay7(nb.ray, (int)q); },
      [&](int64_t q, const RayQueryResult& res) {
        nb.hit[q] = hitRecord(res.hit, res.t, res.prim, res.b1, res.b2);
      });
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(counters + S_CLOSEST, (unsigned long long)n);
}

// traceCam / followCam (SPPM.hs:77-131) for the nodes at tree depth `depth`
template <bool TEX>
__global__ void __launch_bounds__(128, 4) k_sp_camshade(DevAccel A, DevShading S, PassParams P,
                                                        SpCam cs, SpHp hp, const float* __restrict__ r2s,
                                                        int64_t stat_count, int in, int depth, int md,
                                                        unsigned long long* __restrict__ counters) {
  const CamNodes& ni = cs.nb[in];
  const CamNodes& no = cs.nb[1 - in];
  int64_t n = nodeCount(counters, in, cs.NC);
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t nround = (n + stride - 1) / stride * stride;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nround; q += stride) {
    bool rec = false, child[2] = {false, false};
    HitGeom hg;
    DMaterial tm;  // a textured material, resolved at the hit
    float huv[2] = {0.0f, 0.0f};  // its (u, v)
    Bsdf bsdf;
    Spec T;
    Ray ray;
    Ray cray[2];
    Spec cT[2];
    int s = 0, k = 0;
    float sx = 0, sy = 0;
    if (q < n) {
      int2 id = ni.id[q];
      s = id.x;
      k = id.y;
      ray = loadRay7(ni.ray, (int)q);
      T = loadBands(ni.T, (int)q);
      float4 hit = ni.hit[q];
      int prim = __float_as_int(hit.y);
      uint64_t g = P.chunk_base + (uint64_t)s;
      int ix, iy;
      uint32_t sn;
      decodeSample(P, g, ix, iy, sn);
      Sampler smp = mkSampler(P, ix, iy, sn);
      float lu, lv;
      pixelSample(P, smp, ix, iy, sx, sy, lu, lv);
      if (prim == kDegenerateRay) {
        // the reference's sample ends NaN and is dropped by the film
        atomicAdd(counters + S_DEGENERATE, 1ull);
        atomicAdd(cs.Ls + 16 * (size_t)s, NAN);
      } else if (prim < 0) {
        Spec esc = sConst(0.0f);  // escaped: the lights' le (SPPM.hs:74-75)
        for (int l = 0; l < S.n_lights; l++) esc = esc + lightLe(S.lights[l], ray.d);
        Spec L = T * esc;
        if (!isBlack(L)) atomicAddBands(cs.Ls, s, L);
      } else {
        hg = hitGeometry(A, S, ray, prim, hit.x, hit.z, hit.w);
        const DMaterial* mat = S.materials + hg.material;
        if constexpr (TEX) mat = hitMaterial(A, S, ray, prim, hit.x, hit.z, hit.w, hg, tm, huv);
        bsdf = materialBsdf(*mat, hg.n, hg.sp, hg.sn, hg.sdpdu);
        Spec L = T * intLe(S, hg, ray.d);
        if (!isBlack(L)) atomicAddBands(cs.Ls, s, L);
        rec = bsdfHasNonSpecular(bsdf);
        if (depth + 1 < md) {
          V3 wo = -ray.d;
          for (int c = 0; c < 2; c++) {
            uint32_t k2 = 2u * (uint32_t)k + (uint32_t)c;
            uint32_t dim = kDimCamTree + 3u * k2;
            float uc = randF(smp.key, sn, dim), u1 = randF(smp.key, sn, dim + 1),
                  u2 = randF(smp.key, sn, dim + 2);
            BsdfSample bs = sampleBsdfFlags(bsdf, wo, (c ? T_TRANS : T_REFL) | T_SPEC, uc, u1, u2);
            child[c] = !(bs.pdf == 0 || isBlack(bs.f));
            if (child[c]) {
              cray[c] = Ray{bsdf.p, bs.wi, hg.eps, INFINITY};
              cT[c] = bs.f * T;
            }
          }
        }
      }
    }
    long long hpos = appendPos(rec, counters + S_HP);
    if (rec && hpos < (long long)hp.H) {
      int64_t si = statIndex(P, sx, sy);
      float r2 = (si >= 0 && si < stat_count) ? r2s[si] : 0.0f;
      V3 p = bsdf.p, wo = -ray.d;
      hp.p[hpos] = make_float4(p.x, p.y, p.z, r2);
      // the shading geometry after any bump, and (u, v) in the spare lanes
      hp.pix[hpos] = make_float4(sx, sy, __int_as_float(hg.material), huv[0]);
      hp.w[hpos] = make_float4(wo.x, wo.y, wo.z, huv[1]);
      hp.ng[hpos] = make_float4(hg.n.x, hg.n.y, hg.n.z, 0.0f);
      hp.sn[hpos] = make_float4(hg.sn.x, hg.sn.y, hg.sn.z, 0.0f);
      hp.sd[hpos] = make_float4(hg.sdpdu.x, hg.sdpdu.y, hg.sdpdu.z, 0.0f);
      storeBands(hp.F, (int)hpos, T);
    }
    for (int c = 0; c < 2; c++) {
      long long pos = appendPos(child[c], counters + S_NODES0 + (1 - in));
      if (!child[c]) continue;
      if (pos >= (long long)cs.NC) {
        atomicAdd(counters + S_NODE_OVF, 1ull);
        continue;
      }
      storeRay(no.ray, (int)pos, cray[c]);
      storeBands(no.T, (int)pos, cT[c]);
      no.id[pos] = make_int2(s, 2 * k + c);
    }
  }
}

// addSample of every camera sample's gathered emission (SPPM.hs:150-154)
__global__ void __launch_bounds__(128) k_sp_camfilm(PassParams P, SpCam cs, int64_t count,
                                                    float* __restrict__ film, const float* filter,
                                                    unsigned long long* counters) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    splatSampleAt(film, P, P.chunk_base + (uint64_t)i, loadBands(cs.Ls, (int)i),
                  counters + S_NONFINITE, TableFilter{filter});
}

// ------------------------------------------------------------------ spatial hash
// the largest radius^2 and the hit points' position bounds (mkHash)
__global__ void __launch_bounds__(256) k_sp_bounds(SpHp hp, int64_t nh,
                                                   unsigned long long* counters) {
  uint32_t* b = (uint32_t*)counters + kBoundsAt;
  uint32_t r2m = 0, lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0, 0, 0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nh;
       i += (int64_t)gridDim.x * blockDim.x) {
    float4 p = hp.p[i];
    r2m = max(r2m, __float_as_uint(p.w));  // radii^2 are >= 0: their bits order like them
    float c[3] = {p.x, p.y, p.z};
    for (int k = 0; k < 3; k++) {
      lo[k] = min(lo[k], orderedBits(c[k]));
      hi[k] = max(hi[k], orderedBits(c[k]));
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    r2m = max(r2m, __shfl_xor_sync(0xffffffffu, r2m, o));
    for (int k = 0; k < 3; k++) {
      lo[k] = min(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
      hi[k] = max(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(b, r2m);
    for (int k = 0; k < 3; k++) {
      atomicMin(b + 1 + k, lo[k]);
      atomicMax(b + 4 + k, hi[k]);
    }
  }
}

// the cells a hit point's box covers (mkHash, SPPM.hs:324-353); FILL = false
// counts them per bucket, true enters the hit point
template <bool FILL>
__global__ void __launch_bounds__(128) k_sp_cells(SpHp hp, int64_t nh, V3 lo, float invSize,
                                                  long long cnt, uint32_t* __restrict__ counts,
                                                  const uint32_t* __restrict__ off,
                                                  int32_t* __restrict__ entries,
                                                  float4* __restrict__ epos) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nh;
       i += (int64_t)gridDim.x * blockDim.x) {
    float4 p = hp.p[i];
    float r2p = p.w;
    if (r2p == 0) continue;
    float rp = sqrtf(r2p);
    float fx0 = invSize * fabsf((p.x - rp) - lo.x), fy0 = invSize * fabsf((p.y - rp) - lo.y),
          fz0 = invSize * fabsf((p.z - rp) - lo.z);
    float fx1 = invSize * fabsf((p.x + rp) - lo.x), fy1 = invSize * fabsf((p.y + rp) - lo.y),
          fz1 = invSize * fabsf((p.z + rp) - lo.z);
    // cell coordinates beyond 64-bit integers (radii vanishing against the
    // scene) have no defined truncation; such hit points are left out
    if (!(fmaxf(fx1, fmaxf(fy1, fz1)) < 9.2e18f && fmaxf(fx0, fmaxf(fy0, fz0)) < 9.2e18f)) continue;
    long long x0 = (long long)fx0, y0 = (long long)fy0, z0 = (long long)fz0;
    long long x1 = (long long)fx1, y1 = (long long)fy1, z1 = (long long)fz1;
    for (long long x = x0; x <= x1; x++)
      for (long long y = y0; y <= y1; y++)
        for (long long z = z0; z <= z1; z++) {
          long long b = cellBucket(x, y, z, cnt);
          unsigned pos = atomicAdd(counts + b, 1u);
          if (FILL) {
            entries[off[b] + pos] = (int32_t)i;
            epos[off[b] + pos] = p;
          }
        }
  }
}

// exclusive scan of n counts in blocks of 1024 (block sums to sums[])
__global__ void __launch_bounds__(1024) k_scan_blocks(const uint32_t* __restrict__ in,
                                                      uint32_t* __restrict__ out, int64_t n,
                                                      uint32_t* __restrict__ sums) {
  __shared__ uint32_t part[1024];
  int t = threadIdx.x;
  int64_t i = (int64_t)blockIdx.x * 1024 + t;
  uint32_t v = i < n ? in[i] : 0u;
  part[t] = v;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    uint32_t a = t >= o ? part[t - o] : 0u;
    __syncthreads();
    part[t] += a;
    __syncthreads();
  }
  if (i < n) out[i] = part[t] - v;
  if (t == 1023) sums[blockIdx.x] = part[t];
}
// exclusive scan of the block sums in one block; sums[nb] = total
__global__ void __launch_bounds__(1024) k_scan_sums(uint32_t* __restrict__ sums, int64_t nb) {
  __shared__ uint32_t part[1024];
  int t = threadIdx.x;
  int64_t per = (nb + 1023) / 1024;
  uint32_t s = 0;
  for (int64_t k = 0; k < per; k++) {
    int64_t i = t * per + k;
    if (i < nb) s += sums[i];
  }
  part[t] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    uint32_t a = t >= o ? part[t - o] : 0u;
    __syncthreads();
    part[t] += a;
    __syncthreads();
  }
  uint32_t run = part[t] - s;
  for (int64_t k = 0; k < per; k++) {
    int64_t i = t * per + k;
    if (i < nb) {
      uint32_t v = sums[i];
      sums[i] = run;
      run += v;
    }
  }
  if (t == 1023) sums[nb] = part[1023];
}
__global__ void __launch_bounds__(1024) k_scan_add(uint32_t* __restrict__ out, int64_t n,
                                                   const uint32_t* __restrict__ sums) {
  int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
  if (i < n) out[i] += sums[blockIdx.x];
  if (i == 0) out[n] = sums[(n + 1023) / 1024];
}

// ------------------------------------------------------------------ photon pass
// tracePhoton (SPPM.hs:181-193): photons [chunk_base, chunk_base + count)
__global__ void __launch_bounds__(128) k_sp_emit(DevAccel A, DevShading S, PhotonParams Q,
                                                 SpPhotons ph, int64_t count,
                                                 unsigned long long* counters) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t nround = (count + stride - 1) / stride * stride;
  int lc = S.n_lights;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nround; i += stride) {
    bool live = false;
    if (i < count && lc > 0) {
      Sampler smp{pixelKey(Q.seed, Q.pass, 0, 0), (uint32_t)(Q.chunk_base + (uint64_t)i), Q.sn, Q.sn,
                  7, 5};
      float ul = rnd1(smp, 0), uo1, uo2, ud1, ud2;
      rnd2(smp, 0, uo1, uo2);
      rnd2(smp, 1, ud1, ud2);
      int ln = lc == 1 ? 0 : min((int)floorf(ul * (float)lc), lc - 1);
      Spec le;
      Ray ray;
      V3 nl;
      float pdf;
      lightEmit(A, S, S.lights[ln], Q.wc, Q.wr, uo1, uo2, ud1, ud2, le, ray, nl, pdf);
      if (lc != 1) pdf = pdf / (float)lc;
      V3 wi = -ray.d;
      Spec li = sScale(le, absDot(nl, wi) / pdf);
      live = pdf > 0 && !isBlack(li);
      if (live) {
        storeBands(ph.li[0], (int)i, li);
        storeRay(ph.ray, (int)i, ray);
      }
    }
    queueAppend(live, (int)i, ph.live[0], counters + S_PLIVE0);
  }
}

__global__ void k_sp_preset(unsigned long long* counters, int next) {
  if (threadIdx.x == 0) counters[next] = 0;
  if (threadIdx.x == 1) counters[S_NEXT_TRACE] = 0;
}

template <int LAYOUT>
__global__ void __launch_bounds__(128, 8) k_sp_ptrace(DevAccel A, SpPhotons ph, int in,
                                                       unsigned long long* __restrict__ counters) {
  const int32_t* __restrict__ queue = ph.live[in];
  int64_t n = (int64_t)counters[S_PLIVE0 + in];
  traceWarpPersistent<false, LAYOUT, false>(
      A, n, counters + S_NEXT_TRACE, [&](int64_t q) { return loadRay7(ph.ray, queue[q]); },
      [&](int64_t q, const RayQueryResult& res) {
        ph.hit[queue[q]] = hitRecord(res.hit, res.t, res.prim, res.b1, res.b2);
      });
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(counters + S_CLOSEST, (unsigned long long)n);
}

// followPhoton (SPPM.hs:195-243) at photon vertex `depth`: the hit, the
// number of hit points its lookup finds (their splats follow in k_sp_splat)
// and the continuation
template <bool TEX>
__global__ void __launch_bounds__(128, 4) k_sp_vertex(DevAccel A, DevShading S, PhotonParams Q,
                                                      SpPhotons ph, SpHp hp, SpHash hs, int in,
                                                      int depth,
                                                      unsigned long long* __restrict__ counters) {
  const int32_t* __restrict__ qin = ph.live[in];
  const float* __restrict__ li_in = ph.li[depth & 1];
  float* __restrict__ li_out = ph.li[(depth + 1) & 1];
  int64_t n = (int64_t)counters[S_PLIVE0 + in];
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t nround = (n + stride - 1) / stride * stride;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nround; q += stride) {
    bool cont = false, looked = false;
    int s = 0;
    if (q < n) {
      s = qin[q];
      float4 hit = ph.hit[s];
      int prim = __float_as_int(hit.y);
      if (prim == kDegenerateRay) {
        atomicAdd(counters + S_DEGENERATE, 1ull);
      } else if (prim >= 0) {
        Spec li = loadBands(li_in, s);
        Ray ray = loadRay7(ph.ray, s);
        V3 wi = -ray.d;
        HitGeom hg = hitGeometry(A, S, ray, prim, hit.x, hit.z, hit.w);
        DMaterial tm;  // a textured material, resolved at this hit
        const DMaterial* mat = S.materials + hg.material;
        if constexpr (TEX) mat = hitMaterial(A, S, ray, prim, hit.x, hit.z, hit.w, hg, tm);
        Bsdf bsdf = materialBsdf(*mat, hg.n, hg.sp, hg.sn, hg.sdpdu);
        V3 p = bsdf.p;
        long long b = -1;
        if (bsdfHasNonSpecular(bsdf) && hs.cnt > 0) {
          // hashLookup (SPPM.hs:307-314): the bucket of p's cell, scanned by k_sp_count
          float cx = fabsf((p.x - hs.lo.x) * hs.scale), cy = fabsf((p.y - hs.lo.y) * hs.scale),
                cz = fabsf((p.z - hs.lo.z) * hs.scale);
          if (cx < 9.2e18f && cy < 9.2e18f && cz < 9.2e18f)
            b = cellBucket((long long)cx, (long long)cy, (long long)cz, hs.cnt);
        }
        ph.gpos[s] = make_float4(p.x, p.y, p.z, __int_as_float((int)b));
        looked = true;
        ph.gwi[s] = make_float4(wi.x, wi.y, wi.z, absDot(wi, bsdf.ng));
        Sampler smp{pixelKey(Q.seed, Q.pass, 0, 0), (uint32_t)(Q.chunk_base + (uint64_t)s), Q.sn,
                    Q.sn, 7, 5};
        float ubc = rnd1(smp, 1 + depth * 2), u1, u2;
        rnd2(smp, 2 + depth, u1, u2);
        BsdfSample bs = sampleBsdf<true>(bsdf, wi, ubc, u1, u2);
        float pcont = depth > 7 ? 0.8f : 1.0f;
        Spec li2 = sScale(bs.f * li, 1.0f / pcont);
        if (!(bs.pdf == 0 || isBlack(li2)) && !(rnd1(smp, 2 + depth * 2) > pcont)) {
          storeBands(li_out, s, li2);
          storeRay(ph.ray, s, Ray{p, bs.wi, hg.eps, INFINITY});
          cont = true;
        }
      }
      // no hit at all: the count and fill passes skip the entry
      if (!looked) ph.gpos[s] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
    }
    queueAppend(cont, s, ph.live[1 - in], counters + S_PLIVE0 + (1 - in));
  }
}

// the splat of one (photon, hit point) pair: hpF * f * li / (|wi.ng| r^2 pi)
// at the hit point's pixel (splatSample, Image.hs:201-221), and the photon
// count of that pixel
template <bool TEX>
__device__ __forceinline__ void splatPair(const DevShading& S, const PassParams& P,
                                          const SpPhotons& ph, const SpHp& hp, const float* li_in,
                                          int s, int h, float* __restrict__ splat,
                                          uint32_t* __restrict__ m, int64_t stat_count,
                                          unsigned long long* __restrict__ counters) {
  float4 gw = ph.gwi[s];
  V3 wi{gw.x, gw.y, gw.z};
  float4 hpp = hp.p[h], pix = hp.pix[h], w4 = hp.w[h], ng4 = hp.ng[h], sn4 = hp.sn[h], sd4 = hp.sd[h];
  float r2 = hpp.w;
  // the hit point's material: a textured one re-evaluated at its stored
  // shading point and (u, v), its bump already in the stored frame
  int mi = __float_as_int(pix.z);
  DMaterial tm;
  const DMaterial* mat = S.materials + mi;
  if constexpr (TEX)
    if (mat->textured) mat = texturedMaterial(S, mi, TexGeo{V3{hpp.x, hpp.y, hpp.z}, pix.w, w4.w}, tm);
  Bsdf hb = materialBsdf(*mat, V3{ng4.x, ng4.y, ng4.z}, V3{hpp.x, hpp.y, hpp.z},
                         V3{sn4.x, sn4.y, sn4.z}, V3{sd4.x, sd4.y, sd4.z});
  Spec f = evalBsdf<false>(hb, V3{w4.x, w4.y, w4.z}, wi);
  Spec l = sScale(loadBands(hp.F, h) * f * loadBands(li_in, s), 1.0f / (gw.w * r2 * kPi));
  float px = pix.x, py = pix.y;
  if (px >= 0.0f && px < (float)P.width && py >= 0.0f && py < (float)P.height) {
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 16; k++) bad = bad || isnan(l.v[k]) || isinf(l.v[k]);
    if (bad) {
      atomicAdd(counters + S_NONFINITE, 1ull);
    } else {
      float x = 0, y = 0, z = 0;
#pragma unroll
      for (int k = 0; k < 16; k++) {
        x = x + c_cieX[k] * l.v[k];
        y = y + c_cieY[k] * l.v[k];
        z = z + c_cieZ[k] * l.v[k];
      }
      float* o = splat + 3 * ((size_t)floorf(py) * P.width + (size_t)floorf(px));
      atomicAdd(o, x / c_cieYSum);
      atomicAdd(o + 1, y / c_cieYSum);
      atomicAdd(o + 2, z / c_cieYSum);
      atomicAdd(counters + S_SPLATS, 1ull);
    }
  }
  int64_t si = statIndex(P, px, py);
  if (si >= 0 && si < stat_count) atomicAdd(m + si, 1u);
}

// hashLookup/treeLookup (SPPM.hs:307-314, 391-408) with the splats: one warp
// per live photon scans the photon's bucket 32 entries at a time; the hit
// points within their radius go to the warp's queue in shared memory, and
// every 32 queued pairs are splatted by the whole warp (one pair per lane).
constexpr int kGatherBlock = 128;
template <bool TEX>
__global__ void __launch_bounds__(kGatherBlock) k_sp_gather(DevShading S, PassParams P, SpPhotons ph,
                                                            SpHp hp, SpHash hs, int in, int depth,
                                                            float* __restrict__ splat,
                                                            uint32_t* __restrict__ m,
                                                            int64_t stat_count,
                                                            unsigned long long* __restrict__ counters) {
  __shared__ int2 queue[kGatherBlock / 32][64];
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int2* wq = queue[threadIdx.x >> 5];
  const int32_t* __restrict__ qin = ph.live[in];
  const float* __restrict__ li_in = ph.li[depth & 1];
  int64_t n = (int64_t)counters[S_PLIVE0 + in];
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int qn = 0;  // queued pairs (the same in every lane)
  for (int64_t q = warp; q < n; q += nwarps) {
    int s = qin[q];
    float4 gp = ph.gpos[s];
    int b = __float_as_int(gp.w);
    if (b < 0) continue;
    V3 p{gp.x, gp.y, gp.z};
    uint32_t lo = hs.off[b], hi = hs.off[b + 1];
    for (uint32_t e0 = lo; e0 < hi; e0 += 32) {
      uint32_t e = e0 + lane;
      bool found = false;
      if (e < hi) {
        float4 hpp = hs.epos[e];
        found = sqLen(V3{hpp.x, hpp.y, hpp.z} - p) <= hpp.w;
      }
      unsigned mk = __ballot_sync(full, found);
      if (found) wq[qn + __popc(mk & ((1u << lane) - 1))] = make_int2(s, hs.entries[e]);
      qn += __popc(mk);
      __syncwarp();
      if (qn >= 32) {  // a full warp of splats, then the rest to the front of the queue
        int2 pr = wq[lane];
        splatPair<TEX>(S, P, ph, hp, li_in, pr.x, pr.y, splat, m, stat_count, counters);
        __syncwarp();
        int2 rest = lane + 32 < qn ? wq[lane + 32] : make_int2(0, 0);
        __syncwarp();
        if (lane + 32 < qn) wq[lane] = rest;
        qn -= 32;
        __syncwarp();
      }
    }
  }
  if (lane < qn) {
    int2 pr = wq[lane];
    splatPair<TEX>(S, P, ph, hp, li_in, pr.x, pr.y, splat, m, stat_count, counters);
  }
}

// statsUpdate (SPPM.hs:272-295)
__global__ void __launch_bounds__(256) k_sp_stats(SppmPixelStats st, float alpha) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < st.count;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t mm = st.m[i];
    if (mm == 0) continue;
    float r2 = st.r2[i], nn = st.n[i];
    float n2 = nn + alpha * (float)mm;
    float ratio = n2 / (nn + (float)mm);
    st.r2[i] = r2 * ratio;
    st.n[i] = n2;
    st.m[i] = 0;
  }
}

template <class K>
unsigned residentGrid(K kernel, int sms, int block) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
  return (unsigned)(std::max(1, sms) * std::max(1, per_sm));
}

cudaError_t growTo(void*& p, size_t& have, size_t need) {
  if (have >= need && p) return cudaSuccess;
  cudaFree(p);
  p = nullptr;
  have = 0;
  cudaError_t e = cudaMalloc(&p, need);
  if (e == cudaSuccess) have = need;
  return e;
}

// carvers: every array a multiple of 64 entries, so float4 arrays stay aligned
SpCam carveCam(void* base, size_t C, size_t NC) {
  SpCam c;
  float* w = (float*)base;
  c.Ls = w;
  w += 16 * C;
  for (int b = 0; b < 2; b++) {
    c.nb[b].ray = w;
    w += 8 * NC;
    c.nb[b].T = w;
    w += 16 * NC;
    c.nb[b].id = (int2*)w;
    w += 2 * NC;
    c.nb[b].hit = (float4*)w;
    w += 4 * NC;
  }
  c.C = C;
  c.NC = NC;
  return c;
}
size_t camBytes(size_t C, size_t NC) { return 4 * (16 * C + 2 * (8 + 16 + 2 + 4) * NC); }
SpHp carveHp(void* base, size_t H) {
  SpHp h;
  float4* w = (float4*)base;
  h.p = w;
  h.pix = w + H;
  h.w = w + 2 * H;
  h.ng = w + 3 * H;
  h.sn = w + 4 * H;
  h.sd = w + 5 * H;
  h.F = (float*)(w + 6 * H);
  h.H = H;
  return h;
}
size_t hpBytes(size_t H) { return H * (6 * 16 + 64); }
SpPhotons carvePhotons(void* base, size_t cap) {
  SpPhotons p;
  float* w = (float*)base;
  p.li[0] = w;
  w += 16 * cap;
  p.li[1] = w;
  w += 16 * cap;
  p.ray = w;
  w += 8 * cap;
  p.hit = (float4*)w;
  w += 4 * cap;
  p.gpos = (float4*)w;
  w += 4 * cap;
  p.gwi = (float4*)w;
  w += 4 * cap;
  p.live[0] = (int32_t*)w;
  w += cap;
  p.live[1] = (int32_t*)w;
  return p;
}
size_t photonBytes(size_t cap) { return 4 * cap * (16 + 16 + 8 + 4 + 4 + 4 + 2); }

size_t round64(size_t n) { return (std::max<size_t>(n, 64) + 63) / 64 * 64; }

}  // namespace

#define RET_CUDA(call)                                                      \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) {                                                \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);             \
      return e_ == cudaErrorMemoryAllocation ? BLING_ERR_OOM : BLING_ERR_CUDA; \
    }                                                                       \
  } while (0)

void sppm_workspace_free(SppmWorkspace& ws) {
  cudaFree(ws.cam);
  cudaFree(ws.hp);
  cudaFree(ws.buckets);
  cudaFree(ws.entries);
  cudaFree(ws.photons);
  cudaFree(ws.counters);
  ws = SppmWorkspace{};
}

int sppm_extent_pixels(const bling_render_params& rp, int64_t& count, std::string& err) {
  PassParams P;
  int rc = integrator_pass_params(rp, 0, rp.width, rp.height, P, err);
  if (rc) return rc;
  count = (int64_t)P.nx * P.ny;
  return BLING_OK;
}

int sppm_pass(cudaStream_t stream, const DevAccel& A, const DevShading& S, const SppmArgs& a,
              float* d_film, float* d_splat, const SppmPixelStats& px, SppmWorkspace& ws,
              SppmResult& res, std::string& err) {
  res = SppmResult{};
  int device = 0;
  RET_CUDA(cudaGetDevice(&device));
  RET_CUDA(loadCieConstants(device));
  PassParams P;
  int rc = integrator_pass_params(a.rp, 2 * a.pass, a.rp.width, a.rp.height, P, err);
  if (rc) return rc;
  // counters, then the pass's 16x16 filter table
  if (!ws.counters) RET_CUDA(cudaMalloc(&ws.counters, kSpCounterBytes + 256 * sizeof(float)));
  unsigned long long* counters = ws.counters;
  float* d_filter = (float*)((unsigned char*)ws.counters + kSpCounterBytes);
  float tbl[256];
  filterTableHost(a.rp.filter_kind, a.rp.filter_params, P.fw, P.fh, tbl);
  RET_CUDA(cudaMemcpyAsync(d_filter, tbl, sizeof tbl, cudaMemcpyHostToDevice, stream));
  RET_CUDA(cudaMemsetAsync(counters, 0, kSpCounterBytes, stream));
  // device-side copies of three statistics counters around a camera chunk
  auto copyCounter = [&](int to, int from) {
    return cudaMemcpyAsync(counters + to, counters + from, sizeof(unsigned long long),
                           cudaMemcpyDeviceToDevice, stream);
  };
  int sms = 0;
  RET_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int block = 128;
  unsigned g_trace = withLayout(A.wide, [&](auto L) {
    return residentGrid(k_sp_camtrace<decltype(L)::value>, sms, block);
  });
  unsigned g_shade = residentGrid(k_sp_camshade<false>, sms, block);
  unsigned g_wide = (unsigned)std::max(1, sms * 8);

  // ---- 1. camera pass, in chunks of samples; a chunk whose node queue or
  // hit-point buffer overflows is run again with larger buffers
  int64_t total = (int64_t)P.nx * P.ny;  // one sample per pixel of the sample extent
  size_t C = round64((size_t)std::min<int64_t>(total, int64_t(1) << 19));
  size_t NC = std::max(ws.cam_nodes, 4 * C);
  if (ws.cam_samples < C || ws.cam_nodes < NC) {
    size_t have = ws.cam ? camBytes(ws.cam_samples, ws.cam_nodes) : 0;
    RET_CUDA(growTo(ws.cam, have, camBytes(C, NC)));
    ws.cam_samples = C;
    ws.cam_nodes = NC;
  }
  size_t H0 = round64(std::max<size_t>(ws.hp_cap, (size_t)total));
  if (ws.hp_cap < H0) {
    size_t have = ws.hp ? hpBytes(ws.hp_cap) : 0;
    RET_CUDA(growTo(ws.hp, have, hpBytes(H0)));
    ws.hp_cap = H0;
  }
  unsigned long long nh = 0;
  for (int64_t base = 0; base < total;) {
    int64_t count = std::min<int64_t>((int64_t)ws.cam_samples, total - base);
    P.chunk_base = (uint64_t)base;
    SpCam cs = carveCam(ws.cam, ws.cam_samples, ws.cam_nodes);
    SpHp hp = carveHp(ws.hp, ws.hp_cap);
    unsigned cap_blocks = (unsigned)std::max<int64_t>(1, (count + block - 1) / block);
    RET_CUDA(cudaMemcpyAsync(counters + S_HP, &nh, sizeof nh, cudaMemcpyHostToDevice, stream));
    RET_CUDA(cudaMemsetAsync(counters + S_NODE_OVF, 0, sizeof(unsigned long long), stream));
    RET_CUDA(copyCounter(S_SAVED_CLOSEST, S_CLOSEST));
    RET_CUDA(copyCounter(S_SAVED_NONFINITE, S_NONFINITE));
    RET_CUDA(copyCounter(S_SAVED_DEGENERATE, S_DEGENERATE));
    k_sp_camgen<<<std::min(g_wide, cap_blocks), block, 0, stream>>>(P, S.camera, cs, count, counters);
    for (int d = 0; d < a.max_depth; d++) {
      int in = d & 1;
      k_sp_reset<<<1, 32, 0, stream>>>(counters, S_NODES0 + (1 - in));
      unsigned nb = (unsigned)std::max<size_t>(1, (ws.cam_nodes + block - 1) / block);
      withLayout(A.wide, [&](auto L) {
        k_sp_camtrace<decltype(L)::value><<<std::min(g_trace, nb), block, 0, stream>>>(
            A, cs.nb[in], in, cs.NC, counters);
      });
      if (S.textured)
        k_sp_camshade<true><<<std::min(g_shade, nb), block, 0, stream>>>(
            A, S, P, cs, hp, px.r2, px.count, in, d, a.max_depth, counters);
      else
        k_sp_camshade<false><<<std::min(g_shade, nb), block, 0, stream>>>(
            A, S, P, cs, hp, px.r2, px.count, in, d, a.max_depth, counters);
      RET_CUDA(cudaGetLastError());
    }
    unsigned long long c2[S_COUNT];
    RET_CUDA(cudaMemcpyAsync(c2, counters, sizeof c2, cudaMemcpyDeviceToHost, stream));
    RET_CUDA(cudaStreamSynchronize(stream));
    if (c2[S_NODE_OVF] > 0) {  // deeper specular trees than the node queues hold
      size_t NC2 = 2 * ws.cam_nodes;
      if (NC2 > (size_t(1) << 28)) {
        err = "SPPM camera pass: specular branching exceeds the node queue; lower max_depth";
        return BLING_ERR_BOUNDS;
      }
      size_t have = camBytes(ws.cam_samples, ws.cam_nodes);
      RET_CUDA(growTo(ws.cam, have, camBytes(ws.cam_samples, NC2)));
      ws.cam_nodes = NC2;
      RET_CUDA(copyCounter(S_CLOSEST, S_SAVED_CLOSEST));  // the rerun counts afresh
      RET_CUDA(copyCounter(S_NONFINITE, S_SAVED_NONFINITE));
      RET_CUDA(copyCounter(S_DEGENERATE, S_SAVED_DEGENERATE));
      continue;  // run the chunk again
    }
    if (c2[S_HP] > ws.hp_cap) {  // more hit points than the buffer holds: grow, keep the earlier ones
      size_t H2 = round64(2 * (size_t)c2[S_HP]);
      void* nbuf = nullptr;
      RET_CUDA(cudaMalloc(&nbuf, hpBytes(H2)));
      SpHp from = carveHp(ws.hp, ws.hp_cap), to = carveHp(nbuf, H2);
      size_t k = (size_t)nh;
      if (k) {
        RET_CUDA(cudaMemcpyAsync(to.p, from.p, 16 * k, cudaMemcpyDeviceToDevice, stream));
        RET_CUDA(cudaMemcpyAsync(to.pix, from.pix, 16 * k, cudaMemcpyDeviceToDevice, stream));
        RET_CUDA(cudaMemcpyAsync(to.w, from.w, 16 * k, cudaMemcpyDeviceToDevice, stream));
        RET_CUDA(cudaMemcpyAsync(to.ng, from.ng, 16 * k, cudaMemcpyDeviceToDevice, stream));
        RET_CUDA(cudaMemcpyAsync(to.sn, from.sn, 16 * k, cudaMemcpyDeviceToDevice, stream));
        RET_CUDA(cudaMemcpyAsync(to.sd, from.sd, 16 * k, cudaMemcpyDeviceToDevice, stream));
        RET_CUDA(cudaMemcpyAsync(to.F, from.F, 64 * k, cudaMemcpyDeviceToDevice, stream));
      }
      RET_CUDA(cudaStreamSynchronize(stream));
      cudaFree(ws.hp);
      ws.hp = nbuf;
      ws.hp_cap = H2;
      RET_CUDA(copyCounter(S_CLOSEST, S_SAVED_CLOSEST));  // the rerun counts afresh
      RET_CUDA(copyCounter(S_NONFINITE, S_SAVED_NONFINITE));
      RET_CUDA(copyCounter(S_DEGENERATE, S_SAVED_DEGENERATE));
      continue;  // run the chunk again
    }
    k_sp_camfilm<<<std::min(g_wide, cap_blocks), block, 0, stream>>>(P, cs, count, d_film, d_filter,
                                                                       counters);
    RET_CUDA(cudaGetLastError());
    nh = c2[S_HP];
    base += count;
  }
  res.camera_samples = (uint64_t)total;
  res.hitpoints = nh;

  // ---- 2. spatial hash over the hit points (none: the photon pass finds nothing)
  SpHp hp = carveHp(ws.hp, ws.hp_cap);
  SpHash hs{};
  if (nh > 0) {
    uint32_t init[7] = {0, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0, 0, 0};
    RET_CUDA(cudaMemcpyAsync((uint32_t*)counters + kBoundsAt, init, sizeof init,
                             cudaMemcpyHostToDevice, stream));
    k_sp_bounds<<<std::min<unsigned>(g_wide, (unsigned)((nh + 255) / 256)), 256, 0, stream>>>(
        hp, (int64_t)nh, counters);
    uint32_t bb[7];
    RET_CUDA(cudaMemcpyAsync(bb, (uint32_t*)counters + kBoundsAt, sizeof bb, cudaMemcpyDeviceToHost,
                             stream));
    RET_CUDA(cudaStreamSynchronize(stream));
    float r2max;
    memcpy(&r2max, &bb[0], 4);
    float r = sqrtf(r2max);
    V3 pmin{fromOrdered(bb[1]), fromOrdered(bb[2]), fromOrdered(bb[3])};
    V3 lo{pmin.x - r, pmin.y - r, pmin.z - r};
    float invSize = 1.0f / (2.0f * r);
    long long cnt = (long long)nh;
    size_t nblk = ((size_t)cnt + 1023) / 1024;
    size_t words = 2 * ((size_t)cnt + 1) + nblk + 1;  // counts, offsets, block sums
    if (ws.bucket_cap < words) {
      size_t have = ws.buckets ? 4 * ws.bucket_cap : 0;
      RET_CUDA(growTo(ws.buckets, have, 4 * words));
      ws.bucket_cap = words;
    }
    uint32_t* counts = (uint32_t*)ws.buckets;
    uint32_t* off = counts + cnt + 1;
    uint32_t* sums = off + cnt + 1;
    RET_CUDA(cudaMemsetAsync(counts, 0, 4 * ((size_t)cnt + 1), stream));
    unsigned gc = std::min<unsigned>(g_wide, (unsigned)((nh + block - 1) / block));
    k_sp_cells<false><<<gc, block, 0, stream>>>(hp, (int64_t)nh, lo, invSize, cnt, counts, nullptr,
                                                nullptr, nullptr);
    k_scan_blocks<<<(unsigned)nblk, 1024, 0, stream>>>(counts, off, cnt, sums);
    k_scan_sums<<<1, 1024, 0, stream>>>(sums, (int64_t)nblk);
    k_scan_add<<<(unsigned)nblk, 1024, 0, stream>>>(off, cnt, sums);
    RET_CUDA(cudaGetLastError());
    uint32_t E = 0;
    RET_CUDA(cudaMemcpyAsync(&E, off + cnt, 4, cudaMemcpyDeviceToHost, stream));
    RET_CUDA(cudaStreamSynchronize(stream));
    if (ws.entry_cap < (size_t)E + 1) {  // E + 1 positions (float4), then E + 1 indices
      size_t want = round64((size_t)E + 1);
      size_t have = ws.entries ? 20 * ws.entry_cap : 0;
      RET_CUDA(growTo(ws.entries, have, 20 * want));
      ws.entry_cap = want;
    }
    float4* epos = (float4*)ws.entries;
    int32_t* eidx = (int32_t*)(epos + ws.entry_cap);
    RET_CUDA(cudaMemsetAsync(counts, 0, 4 * ((size_t)cnt + 1), stream));
    k_sp_cells<true><<<gc, block, 0, stream>>>(hp, (int64_t)nh, lo, invSize, cnt, counts, off,
                                               eidx, epos);
    RET_CUDA(cudaGetLastError());
    hs = SpHash{lo, invSize, cnt, off, eidx, epos};
  }

  // ---- 3. photon pass
  int sn = std::max(1, (int)ceilf(sqrtf((float)a.photons)));
  int64_t nphot = (int64_t)sn * sn;
  res.photons = (uint64_t)nphot;
  if (nh > 0 && S.n_lights > 0) {
    size_t cap = round64((size_t)std::min<int64_t>(nphot, int64_t(1) << 20));
    if (ws.photon_cap < cap) {
      size_t have = ws.photons ? photonBytes(ws.photon_cap) : 0;
      RET_CUDA(growTo(ws.photons, have, photonBytes(cap)));
      ws.photon_cap = cap;
    }
    SpPhotons ph = carvePhotons(ws.photons, ws.photon_cap);
    PhotonParams Q;
    Q.seed = a.seed;
    Q.pass = 2 * a.pass + 1;
    Q.sn = sn;
    Q.wc = V3{a.wc[0], a.wc[1], a.wc[2]};
    Q.wr = a.wr;
    unsigned g_pt = withLayout(A.wide, [&](auto L) {
      return residentGrid(k_sp_ptrace<decltype(L)::value>, sms, block);
    });
    unsigned g_vx = residentGrid(k_sp_vertex<false>, sms, block);
    for (int64_t base = 0; base < nphot; base += (int64_t)ws.photon_cap) {
      int64_t count = std::min<int64_t>((int64_t)ws.photon_cap, nphot - base);
      Q.chunk_base = (uint64_t)base;
      unsigned emit_blocks = (unsigned)std::max<int64_t>(1, (count + block - 1) / block);
      k_sp_preset<<<1, 32, 0, stream>>>(counters, S_PLIVE0);
      k_sp_emit<<<std::min(g_wide, emit_blocks), block, 0, stream>>>(A, S, Q, ph, count, counters);
      RET_CUDA(cudaGetLastError());
      int64_t n_cur = count;  // an upper bound of the live photons, exact after the first bounce
      for (int depth = 0;; depth++) {
        int in = depth & 1;
        unsigned cap_blocks = (unsigned)std::max<int64_t>(1, (n_cur + block - 1) / block);
        k_sp_preset<<<1, 32, 0, stream>>>(counters, S_PLIVE0 + (1 - in));
        withLayout(A.wide, [&](auto L) {
          k_sp_ptrace<decltype(L)::value><<<std::min(g_pt, cap_blocks), block, 0, stream>>>(
              A, ph, in, counters);
        });
        unsigned warp_blocks = (unsigned)std::max<int64_t>(1, (n_cur + 3) / 4);  // 4 warps a block
        if (S.textured) {
          k_sp_vertex<true><<<std::min(g_vx, cap_blocks), block, 0, stream>>>(
              A, S, Q, ph, hp, hs, in, depth, counters);
          k_sp_gather<true><<<std::min(g_wide * 2, warp_blocks), kGatherBlock, 0, stream>>>(
              S, P, ph, hp, hs, in, depth, d_splat, px.m, px.count, counters);
        } else {
          k_sp_vertex<false><<<std::min(g_vx, cap_blocks), block, 0, stream>>>(
              A, S, Q, ph, hp, hs, in, depth, counters);
          k_sp_gather<false><<<std::min(g_wide * 2, warp_blocks), kGatherBlock, 0, stream>>>(
              S, P, ph, hp, hs, in, depth, d_splat, px.m, px.count, counters);
        }
        RET_CUDA(cudaGetLastError());
        unsigned long long live = (unsigned long long)n_cur;
        if (depth >= 3 && (depth & 3) == 3) {  // the live count, every fourth bounce
          RET_CUDA(cudaMemcpyAsync(&live, counters + S_PLIVE0 + (1 - in), sizeof live,
                                   cudaMemcpyDeviceToHost, stream));
          RET_CUDA(cudaStreamSynchronize(stream));
        }
        if (live == 0) break;
        n_cur = (int64_t)live;
      }
    }
  }

  // ---- 4. radius update
  k_sp_stats<<<std::min<unsigned>(g_wide, (unsigned)((px.count + 255) / 256 + 1)), 256, 0, stream>>>(
      px, a.alpha);
  RET_CUDA(cudaGetLastError());
  unsigned long long cnt[S_COUNT];
  RET_CUDA(cudaMemcpyAsync(cnt, counters, sizeof cnt, cudaMemcpyDeviceToHost, stream));
  RET_CUDA(cudaStreamSynchronize(stream));
  res.rays_closest = cnt[S_CLOSEST];
  res.splats = cnt[S_SPLATS];
  res.nonfinite = cnt[S_NONFINITE];
  res.degenerate = cnt[S_DEGENERATE];
  return BLING_OK;
}

}  // namespace bgpu
