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
//   k_trace         closest hit of the bounce rays (scIntersect)
//   k_shade         emission on specular paths, the BSDF, one light sample and
//                   one BSDF sample for MIS (sampleOneLight/estimateDirect,
//                   Scene.hs:184-241), Russian roulette and the continuation
//                   sample; queues the shadow ray, the MIS ray and the vertex
//   k_trace_shadow  any hit of the shadow rays (occluded)
//   k_trace_mis     closest hit of the MIS rays
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
#include <vector>

#include "filter_host.h"
#include "integrator_device.cuh"

namespace bgpu {

// ------------------------------------------------------------------ slot state
enum : int { VF_SHADOW = 1, VF_MIS = 2, VF_CONT = 4 };

struct Slots {
  size_t cap;
  float* T;          // 16 x cap
  float* L;          // 16 x cap
  float* ray;        // 7 x cap: o, d, tmin (sign bit of tmin: the previous bounce was specular)
  float* hit_t;      // cap
  int32_t* hit_prim; // cap
  float* hit_b;      // 2 x cap
  // the current vertex, deferred until its shadow and MIS rays are traced
  float* intl;       // 16 x cap: emission seen on a specular path
  float* ls;         // 16 x cap: light-sample term before visibility
  float* bsf;        // 16 x cap: MIS BSDF sample throughput
  float* fc;         // 16 x cap: continuation BSDF sample throughput
  float* bsw;        // cap: MIS weight of the BSDF sample
  float* invpc;      // cap: 1 / continuation probability
  int32_t* vflags;   // cap: VF_* | light index << 8
  float* sray;       // 8 x cap: shadow ray o, d, tmin, tmax
  int32_t* svis;     // cap: shadow ray unoccluded
  float* mray;       // 7 x cap: MIS ray o, d, tmin
  float* mhit_t;     // cap
  int32_t* mhit_prim;// cap
  float* mhit_b;     // 2 x cap
};

struct Queues {
  int32_t* live[2];  // paths to trace this bounce / next bounce
  int32_t* shadow;
  int32_t* mis;
  int32_t* resolve;
};

// counters (unsigned long long): queue sizes and statistics
enum : int {
  C_LIVE0 = 0, C_LIVE1 = 1, C_CLOSEST = 2, C_ANY = 3, C_NONFINITE = 4, C_NEXT_TRACE = 5,
  C_SHADOW = 6, C_MIS = 7, C_RESOLVE = 8, C_NEXT_SHADOW = 9, C_NEXT_MIS = 10, C_DEGENERATE = 11,
  C_COUNT = 16
};

constexpr size_t kSlotWords = 16 * 6 + 7 + 4 + 3 + 8 + 1 + 7 + 4;  // per slot, 4-byte words
constexpr size_t kQueueWords = 5;
constexpr size_t kCounterBytes = 256;

static size_t slotBytes(size_t cap) { return kCounterBytes + (kSlotWords + kQueueWords) * 4 * cap; }

// lays slots, queues and counters out in one buffer of slotBytes(cap) bytes
static void carve(unsigned char* base, size_t cap, Slots& st, Queues& q,
                  unsigned long long*& counters) {
  counters = (unsigned long long*)base;
  float* w = (float*)(base + kCounterBytes);
  auto take = [&](size_t words) {
    float* p = w;
    w += words * cap;
    return p;
  };
  st.cap = cap;
  st.T = take(16);
  st.L = take(16);
  st.ray = take(7);
  st.hit_t = take(1);
  st.hit_prim = (int32_t*)take(1);
  st.hit_b = take(2);
  st.intl = take(16);
  st.ls = take(16);
  st.bsf = take(16);
  st.fc = take(16);
  st.bsw = take(1);
  st.invpc = take(1);
  st.vflags = (int32_t*)take(1);
  st.sray = take(8);
  st.svis = (int32_t*)take(1);
  st.mray = take(7);
  st.mhit_t = take(1);
  st.mhit_prim = (int32_t*)take(1);
  st.mhit_b = take(2);
  q.live[0] = (int32_t*)take(1);
  q.live[1] = (int32_t*)take(1);
  q.shadow = (int32_t*)take(1);
  q.mis = (int32_t*)take(1);
  q.resolve = (int32_t*)take(1);
}

__device__ __forceinline__ void decodeSample(const PassParams& P, uint64_t g, int& ix, int& iy,
                                             uint32_t& n) {
  uint64_t pix = g / (uint64_t)P.spp;
  n = (uint32_t)(g % (uint64_t)P.spp);
  ix = P.x0 + (int)(pix % (uint64_t)P.nx);
  iy = P.y0 + (int)(pix / (uint64_t)P.nx);
}
__device__ __forceinline__ Sampler mkSampler(const PassParams& P, int ix, int iy, uint32_t n) {
  Sampler s;
  s.key = pixelKey(P.seed, P.pass, ix, iy);
  s.n = n;
  s.nu = P.nu;
  s.nv = P.nv;
  s.n1d = P.n1d;
  s.n2d = P.n2d;
  return s;
}
__device__ __forceinline__ void pixelSample(const PassParams& P, const Sampler& s, int ix, int iy,
                                            float& sx, float& sy, float& lu, float& lv) {
  float ox, oy;
  strat2D(s, s.n, DIM_PIX_U, DIM_PIX_V, ox, oy);
  uint32_t N = (uint32_t)P.spp;
  uint32_t lp = permute(s.n, N, randU32(s.key, 0xffffffffu, DIM_LENS_PERM));
  strat2D(s, lp, DIM_LENS_U, DIM_LENS_V, lu, lv);
  sx = (float)ix + ox;
  sy = (float)iy + oy;
}

__device__ __forceinline__ Spec loadBands(const float* base, size_t cap, int s) {
  Spec v;
#pragma unroll
  for (int b = 0; b < 16; b++) v.v[b] = base[b * cap + s];
  return v;
}
__device__ __forceinline__ void storeBands(float* base, size_t cap, int s, const Spec& v) {
#pragma unroll
  for (int b = 0; b < 16; b++) base[b * cap + s] = v.v[b];
}
__device__ __forceinline__ void storeRay(float* base, size_t cap, int s, const Ray& r, bool tmax) {
  base[s] = r.o.x;
  base[cap + s] = r.o.y;
  base[2 * cap + s] = r.o.z;
  base[3 * cap + s] = r.d.x;
  base[4 * cap + s] = r.d.y;
  base[5 * cap + s] = r.d.z;
  base[6 * cap + s] = r.tmin;
  if (tmax) base[7 * cap + s] = r.tmax;
}
__device__ __forceinline__ Ray loadRay7(const float* base, size_t cap, int s) {
  return Ray{V3{base[s], base[cap + s], base[2 * cap + s]},
             V3{base[3 * cap + s], base[4 * cap + s], base[5 * cap + s]}, fabsf(base[6 * cap + s]),
             INFINITY};
}

// warp-aggregated append (every lane of the warp calls it)
__device__ __forceinline__ void queueAppend(bool live, int slot, int32_t* __restrict__ queue,
                                            unsigned long long* count) {
  const unsigned mask = 0xffffffffu;
  __syncwarp();
  unsigned ballot = __ballot_sync(mask, live);
  if (!ballot) return;
  int lane = threadIdx.x & 31;
  int leader = __ffs(ballot) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(count, (unsigned long long)__popc(ballot));
  base = __shfl_sync(mask, base, leader);
  if (live) queue[base + __popc(ballot & ((1u << lane) - 1))] = slot;
}

// intLe (Primitive.hs:68-76) + lEmit (Light.hs:85-96)
__device__ __forceinline__ Spec intLe(const DevShading& S, const HitGeom& g, V3 wo) {
  if (g.light_id < 0) return sConst(0);
  return dot(g.n, wo) > 0 ? sLoad(S.shape_emission + 16 * g.shape) : sConst(0);
}

// ------------------------------------------------------------------ kernels
// camera rays (fireRay, Camera.hs:146-164) for samples [chunk_base, chunk_base + count)
__global__ void k_raygen(PassParams P, bling_camera_desc cam, Slots st, int64_t count,
                         int32_t* __restrict__ queue, unsigned long long* counters) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t g = P.chunk_base + (uint64_t)i;
    int ix, iy;
    uint32_t n;
    decodeSample(P, g, ix, iy, n);
    Sampler s = mkSampler(P, ix, iy, n);
    float sx, sy, lu, lv;
    pixelSample(P, s, ix, iy, sx, sy, lu, lv);
    V3 pCamera = transPoint(cam.r2c, V3{sx, sy, 0});
    Ray ray{V3{0, 0, 0}, normalize(pCamera), 0, INFINITY};
    if (cam.lens_radius > 0) {
      float u, v;
      concentricSampleDisk(lu, lv, u, v);
      V3 ro{u * cam.lens_radius, v * cam.lens_radius, 0};
      V3 pFocus = rayAt(ray, cam.focal_distance / ray.d.z);
      ray = Ray{ro, normalize(pFocus - ro), 0, INFINITY};
    }
    ray = transRay(cam.c2w, ray);
    storeRay(st.ray, st.cap, (int)i, ray, false);
    storeBands(st.T, st.cap, (int)i, sConst(1.0f));
    storeBands(st.L, st.cap, (int)i, sConst(0.0f));
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
  if (t == 3) counters[C_MIS] = 0;
  if (t == 4) counters[C_RESOLVE] = 0;
  if (t == 5) counters[C_NEXT_SHADOW] = 0;
  if (t == 6) counters[C_NEXT_MIS] = 0;
}

// closest hit of the live paths' rays (scIntersect)
template <bool WIDE>
__global__ void __launch_bounds__(128) k_trace(DevAccel A, Slots st, const int32_t* __restrict__ queue,
                                               const unsigned long long* __restrict__ qcount,
                                               unsigned long long* __restrict__ counters) {
  int64_t n = (int64_t)*qcount;
  traceWarpPersistent<false, WIDE, false>(
      A, n, counters + C_NEXT_TRACE, [&](int64_t q) { return loadRay7(st.ray, st.cap, queue[q]); },
      [&](int64_t q, const RayQueryResult& res) {
        int s = queue[q];
        st.hit_t[s] = res.t;
        st.hit_prim[s] = res.hit ? res.prim : -1;
        st.hit_b[2 * s] = res.b1;
        st.hit_b[2 * s + 1] = res.b2;
      });
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(counters + C_CLOSEST, (unsigned long long)n);
}

// occlusion of the shadow rays (occluded, Scene.hs:168-170)
template <bool WIDE>
__global__ void __launch_bounds__(128) k_trace_shadow(DevAccel A, Slots st,
                                                      const int32_t* __restrict__ queue,
                                                      unsigned long long* __restrict__ counters) {
  int64_t n = (int64_t)counters[C_SHADOW];
  traceWarpPersistent<true, WIDE, false>(
      A, n, counters + C_NEXT_SHADOW,
      [&](int64_t q) {
        int s = queue[q];
        size_t c = st.cap;
        return Ray{V3{st.sray[s], st.sray[c + s], st.sray[2 * c + s]},
                   V3{st.sray[3 * c + s], st.sray[4 * c + s], st.sray[5 * c + s]},
                   st.sray[6 * c + s], st.sray[7 * c + s]};
      },
      [&](int64_t q, const RayQueryResult& res) {
        st.svis[queue[q]] = res.hit ? 0 : 1;
        if (res.prim == kDegenerateRay) atomicAdd(counters + C_DEGENERATE, 1ull);
      });
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(counters + C_ANY, (unsigned long long)n);
}

// closest hit of the BSDF-sampled MIS rays
template <bool WIDE>
__global__ void __launch_bounds__(128) k_trace_mis(DevAccel A, Slots st,
                                                   const int32_t* __restrict__ queue,
                                                   unsigned long long* __restrict__ counters) {
  int64_t n = (int64_t)counters[C_MIS];
  traceWarpPersistent<false, WIDE, false>(
      A, n, counters + C_NEXT_MIS, [&](int64_t q) { return loadRay7(st.mray, st.cap, queue[q]); },
      [&](int64_t q, const RayQueryResult& res) {
        int s = queue[q];
        st.mhit_t[s] = res.t;
        st.mhit_prim[s] = res.hit ? res.prim : -1;
        st.mhit_b[2 * s] = res.b1;
        st.mhit_b[2 * s + 1] = res.b2;
      });
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(counters + C_CLOSEST, (unsigned long long)n);
}

// the splat of a finished path (the raster position is recomputed from the sampler)
__device__ __forceinline__ void finishPath(float* film, const PassParams& P, int slot,
                                           const Spec& L, unsigned long long* counters) {
  uint64_t g = P.chunk_base + (uint64_t)slot;  // slots never move
  int ix, iy;
  uint32_t sn;
  decodeSample(P, g, ix, iy, sn);
  Sampler smp = mkSampler(P, ix, iy, sn);
  float sx, sy, lu, lv;
  pixelSample(P, smp, ix, iy, sx, sy, lu, lv);
  filmAdd(film, P, ix, iy, sx, sy, L, counters + C_NONFINITE);
}

// one vertex of every live path, up to its shadow and MIS rays (Path.hs:49-87)
__global__ void __launch_bounds__(128) k_shade(DevAccel A, DevShading S, PassParams P, Slots st,
                                               Queues Q, int depth, int live_in,
                                               float* __restrict__ film,
                                               unsigned long long* __restrict__ counters) {
  int64_t n = (int64_t)counters[live_in];
  const int32_t* __restrict__ qin = Q.live[live_in];
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t nround = (n + stride - 1) / stride * stride;  // whole warps stay together for the appends
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nround; q += stride) {
    bool want_shadow = false, want_mis = false, want_resolve = false;
    int s = 0;
    if (q < n) {
      s = qin[q];
      uint64_t g = P.chunk_base + (uint64_t)s;
      int ix, iy;
      uint32_t sn;
      decodeSample(P, g, ix, iy, sn);
      Sampler smp = mkSampler(P, ix, iy, sn);
      size_t c = st.cap;
      Ray ray = loadRay7(st.ray, c, s);
      bool specular = depth == 0 || signbit(st.ray[6 * c + s]);
      int prim = st.hit_prim[s];
      if (prim == kDegenerateRay) {
        // a NaN ray: the reference's sample ends NaN and is dropped by the film
        atomicAdd(counters + C_DEGENERATE, 1ull);
        finishPath(film, P, s, sConst(NAN), counters);
      } else if (prim < 0 || depth == P.max_depth) {
        Spec Lr = loadBands(st.L, c, s);
        if (prim < 0 && specular) {  // nothing hit after a specular bounce: l + t * sum le
          Spec sum = sConst(0);
          for (int k = 0; k < S.n_lights; k++) sum = sum + lightLe(S.lights[k], ray.d);
          Lr = Lr + loadBands(st.T, c, s) * sum;
        }
        finishPath(film, P, s, Lr, counters);
      } else {
        float thit = st.hit_t[s], b1 = st.hit_b[2 * s], b2 = st.hit_b[2 * s + 1];
        float lNumU = rnd1(smp, 1 + 4 * depth);
        float ld1, ld2;
        rnd2(smp, 1 + 3 * depth, ld1, ld2);
        float lBsdfCompU = rnd1(smp, 2 + 4 * depth);
        float lb1, lb2;
        rnd2(smp, 2 + 3 * depth, lb1, lb2);
        HitGeom gm = hitGeometry(A, S, ray, prim, thit, b1, b2);
        V3 rd = ray.d;
        storeBands(st.intl, c, s, specular ? intLe(S, gm, rd) : sConst(0));
        V3 wo = -rd;
        Bsdf bsdf = materialBsdf(S.materials, gm.material, gm.n, gm.sp, gm.sn, gm.sdpdu);
        V3 nn = bsdf.cs.n, p = bsdf.p;
        float eps = gm.eps;
        int flags = 0;
        int lc = S.n_lights;
        int ln = 0;
        if (lc > 0) {
          // sampleOneLight (Scene.hs:233-241) -> estimateDirect (Scene.hs:218-222)
          if (lc > 1) ln = min((int)floorf(lNumU * (float)lc), lc - 1);
          const DLight& l = S.lights[ln];
          // sampleLightMis (Scene.hs:184-192), visibility deferred
          LightSample smpl = lightSample(A, S, l, p, eps, nn, ld1, ld2);
          if (!(smpl.pdf == 0 || isBlack(smpl.li))) {
            Spec f = evalBsdf(bsdf, wo, smpl.wi);
            if (!isBlack(f)) {
              Spec lsv;
              if (smpl.delta) {
                lsv = sScale(f * smpl.li, 1.0f / smpl.pdf);
              } else {
                float w = powerHeuristic(smpl.pdf, bsdfPdf(bsdf, wo, smpl.wi));
                lsv = sScale(f * smpl.li, w / smpl.pdf);
              }
              storeBands(st.ls, c, s, lsv);
              Ray sr = smpl.ray;
              storeRay(st.sray, c, s, sr, true);
              flags |= VF_SHADOW;
            }
          }
          // sampleBsdfMis (Scene.hs:194-205), the hit deferred
          BsdfSample bm = sampleBsdf(bsdf, wo, lBsdfCompU, lb1, lb2);
          if (!(bm.pdf == 0 || isBlack(bm.f))) {
            storeBands(st.bsf, c, s, bm.f);
            st.bsw[s] = powerHeuristic(bm.pdf, lightPdf(A, l, p, bm.wi));
            storeRay(st.mray, c, s, Ray{p, bm.wi, eps, INFINITY}, false);
            flags |= VF_MIS;
          }
        }
        // Russian roulette and the continuation (Path.hs:68-87)
        Spec T = loadBands(st.T, c, s);
        float pc = depth <= P.rr_depth ? 1.0f : hmin(0.75f, sY(T));
        float x = rnd1(smp, 3 + 4 * depth);
        if (!(x > pc)) {
          float uc = rnd1(smp, 0 + 4 * depth);
          float ud1, ud2;
          rnd2(smp, 0 + 3 * depth, ud1, ud2);
          BsdfSample bc = sampleBsdf(bsdf, wo, uc, ud1, ud2);
          if (!(bc.pdf == 0 || isBlack(bc.f))) {
            storeBands(st.fc, c, s, bc.f);
            st.invpc[s] = 1.0f / pc;
            bool spec2 = (bc.type & T_SPEC) != 0;
            storeRay(st.ray, c, s, Ray{p, bc.wi, spec2 ? -eps : eps, INFINITY}, false);
            flags |= VF_CONT;
          }
        }
        st.vflags[s] = flags | (ln << 8);
        want_shadow = (flags & VF_SHADOW) != 0;
        want_mis = (flags & VF_MIS) != 0;
        want_resolve = true;
      }
    }
    queueAppend(want_shadow, s, Q.shadow, counters + C_SHADOW);
    queueAppend(want_mis, s, Q.mis, counters + C_MIS);
    queueAppend(want_resolve, s, Q.resolve, counters + C_RESOLVE);
  }
}

// the vertex's radiance and the continuation (Path.hs:60-87)
__global__ void __launch_bounds__(128) k_resolve(DevAccel A, DevShading S, PassParams P, Slots st,
                                                 Queues Q, int live_out, float* __restrict__ film,
                                                 unsigned long long* __restrict__ counters) {
  int64_t n = (int64_t)counters[C_RESOLVE];
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t nround = (n + stride - 1) / stride * stride;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nround; q += stride) {
    bool cont = false;
    int s = 0;
    if (q < n) {
      s = Q.resolve[q];
      size_t c = st.cap;
      int vf = st.vflags[s];
      int lc = S.n_lights;
      Spec ed = sConst(0);  // estimateDirect = ls + bs (Scene.hs:218)
      Spec lsv = sConst(0), bsv = sConst(0);
      if ((vf & VF_SHADOW) && st.svis[s]) lsv = loadBands(st.ls, c, s);
      if (vf & VF_MIS) {
        const DLight& l = S.lights[vf >> 8];
        Ray mr = loadRay7(st.mray, c, s);
        int mp = st.mhit_prim[s];
        bool use = false;
        Spec lr;
        if (mp == kDegenerateRay) {
          atomicAdd(counters + C_DEGENERATE, 1ull);
          lr = sConst(NAN);  // a NaN ray poisons the sample, which the film then drops
          use = true;
        } else if (mp >= 0) {
          if (l.kind == DLIGHT_AREA) {
            int2 info = __ldg(S.prim_info + mp);
            if (info.x < 0 && ~info.x == l.shape) {  // Eq Light: the same area light
              HitGeom gm = hitGeometry(A, S, mr, mp, st.mhit_t[s], st.mhit_b[2 * s],
                                       st.mhit_b[2 * s + 1]);
              lr = intLe(S, gm, -mr.d);
              use = true;
            }
          }
        } else {
          lr = lightLe(l, mr.d);
          use = true;
        }
        if (use) bsv = sScale(loadBands(st.bsf, c, s) * lr, st.bsw[s]);
      }
      ed = lsv + bsv;
      Spec direct = lc == 1 ? ed : (lc > 1 ? sScale(ed, (float)lc) : sConst(0));
      Spec lHere = loadBands(st.intl, c, s) + direct;
      Spec T = loadBands(st.T, c, s);
      Spec Lr = loadBands(st.L, c, s) + T * lHere;
      if (vf & VF_CONT) {
        storeBands(st.T, c, s, sScale(loadBands(st.fc, c, s) * T, st.invpc[s]));
        storeBands(st.L, c, s, Lr);
        cont = true;
      } else {
        finishPath(film, P, s, Lr, counters);
      }
    }
    queueAppend(cont, s, Q.live[live_out], counters + live_out);
  }
}

// ------------------------------------------------------------------ host side
namespace {

bool g_const_ready[64] = {false};

float fbitsHost(uint32_t b) {
  float f;
  memcpy(&f, &b, 4);
  return f;
}

cudaError_t ensureConstants(int device) {
  if (device >= 0 && device < 64 && g_const_ready[device]) return cudaSuccess;
  float x[16], y[16], z[16];
  for (int i = 0; i < 16; i++) {
    x[i] = fbitsHost(BLING_CIE_X_BITS[i]);
    y[i] = fbitsHost(BLING_CIE_Y_BITS[i]);
    z[i] = fbitsHost(BLING_CIE_Z_BITS[i]);
  }
  float ys = fbitsHost(BLING_CIE_Y_SUM_BITS);
  cudaError_t e;
  if ((e = cudaMemcpyToSymbol(c_cieX, x, sizeof x)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_cieY, y, sizeof y)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_cieZ, z, sizeof z)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_cieYSum, &ys, sizeof ys)) != cudaSuccess) return e;
  if (device >= 0 && device < 64) g_const_ready[device] = true;
  return cudaSuccess;
}

template <class K>
unsigned residentGrid(K kernel, int sms) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0);
  return (unsigned)(std::max(1, sms) * std::max(1, per_sm));
}

struct Grids {
  unsigned trace, shadow, mis, shade, resolve, raygen;
};
Grids g_grids[64];
bool g_grids_ready[64] = {false};

Grids grids(int device, int sms) {
  if (device >= 0 && device < 64 && g_grids_ready[device]) return g_grids[device];
  Grids g;
  // both layouts' kernels use the same registers within a few; take the smaller grid
  g.trace = std::min(residentGrid(k_trace<true>, sms), residentGrid(k_trace<false>, sms));
  g.shadow = std::min(residentGrid(k_trace_shadow<true>, sms), residentGrid(k_trace_shadow<false>, sms));
  g.mis = std::min(residentGrid(k_trace_mis<true>, sms), residentGrid(k_trace_mis<false>, sms));
  g.shade = residentGrid(k_shade, sms);
  g.resolve = residentGrid(k_resolve, sms);
  g.raygen = (unsigned)std::max(1, sms * 8);
  if (device >= 0 && device < 64) {
    g_grids[device] = g;
    g_grids_ready[device] = true;
  }
  return g;
}

// the pass constants (imageWindow', Image.hs:170-176; Path.hs:34-36)
int passParams(const bling_render_params& p, uint64_t pass, int fw, int fh, PassParams& P,
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
  P.n1d = 4 * p.sample_depth;
  P.n2d = 3 * p.sample_depth;
  P.max_depth = p.max_depth;
  P.rr_depth = p.rr_depth;
  P.width = fw;
  P.height = fh;
  return BLING_OK;
}

// the bounces of one chunk of path samples
cudaError_t runChunk(cudaStream_t stream, const DevAccel& A, const DevShading& S, PassParams P,
                     Slots st, Queues Q, unsigned long long* counters, int64_t count, int max_depth,
                     float* d_film, const Grids& G) {
  const int block = 128;
  unsigned g_ray = (unsigned)std::min<int64_t>((count + block - 1) / block, (int64_t)G.raygen);
  k_raygen<<<g_ray, block, 0, stream>>>(P, S.camera, st, count, Q.live[0], counters);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  unsigned cap_blocks = (unsigned)std::max<int64_t>(1, (count + block - 1) / block);
  for (int depth = 0; depth <= max_depth; depth++) {
    int in = depth & 1;
    k_bounce_reset<<<1, 32, 0, stream>>>(counters, C_LIVE0 + (1 - in));
    unsigned gt = std::min(G.trace, cap_blocks), gs = std::min(G.shadow, cap_blocks),
             gm = std::min(G.mis, cap_blocks);
    if (A.wide)
      k_trace<true><<<gt, block, 0, stream>>>(A, st, Q.live[in], counters + C_LIVE0 + in, counters);
    else
      k_trace<false><<<gt, block, 0, stream>>>(A, st, Q.live[in], counters + C_LIVE0 + in, counters);
    k_shade<<<std::min(G.shade, cap_blocks), block, 0, stream>>>(A, S, P, st, Q, depth,
                                                                  C_LIVE0 + in, d_film, counters);
    if (A.wide) {
      k_trace_shadow<true><<<gs, block, 0, stream>>>(A, st, Q.shadow, counters);
      k_trace_mis<true><<<gm, block, 0, stream>>>(A, st, Q.mis, counters);
    } else {
      k_trace_shadow<false><<<gs, block, 0, stream>>>(A, st, Q.shadow, counters);
      k_trace_mis<false><<<gm, block, 0, stream>>>(A, st, Q.mis, counters);
    }
    k_resolve<<<std::min(G.resolve, cap_blocks), block, 0, stream>>>(A, S, P, st, Q,
                                                                      C_LIVE0 + (1 - in), d_film,
                                                                      counters);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

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

static int ensureWorkspace(IntegratorWorkspace& ws, size_t cap, std::string& err) {
  if (ws.capacity >= cap && ws.buffer) return BLING_OK;
  integrator_workspace_free(ws);
  RET_CUDA(cudaMalloc(&ws.buffer, slotBytes(cap)));
  ws.capacity = cap;
  return BLING_OK;
}

int integrator_render_pass(cudaStream_t stream, const DevAccel& A, const DevShading& S,
                           const bling_render_params& p, uint64_t pass, float* d_film, int fw,
                           int fh, IntegratorWorkspace& ws, PassResult& res, std::string& err) {
  int device = 0;
  RET_CUDA(cudaGetDevice(&device));
  RET_CUDA(ensureConstants(device));
  PassParams P;
  int rc = passParams(p, pass, fw, fh, P, err);
  if (rc) return rc;
  uint64_t total = (uint64_t)P.nx * P.ny * P.spp;
  if (total >= (uint64_t(1) << 40)) {
    err = "too many samples in one pass";
    return BLING_ERR_INVALID_ARG;
  }
  float tbl[256];
  filterTableHost(p.filter_kind, p.filter_params, P.fw, P.fh, tbl);
  RET_CUDA(cudaMemcpyToSymbolAsync(c_filter, tbl, sizeof tbl, 0, cudaMemcpyHostToDevice, stream));
  size_t cap = (size_t)std::min<uint64_t>(total, uint64_t(1) << 22);
  rc = ensureWorkspace(ws, std::max<size_t>(cap, 1024), err);
  if (rc) return rc;
  Slots st;
  Queues Q;
  unsigned long long* counters;
  carve((unsigned char*)ws.buffer, ws.capacity, st, Q, counters);
  RET_CUDA(cudaMemsetAsync(counters, 0, C_COUNT * sizeof(unsigned long long), stream));
  int sms = 0;
  RET_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  Grids G = grids(device, sms);
  for (uint64_t base = 0; base < total; base += ws.capacity) {
    int64_t count = (int64_t)std::min<uint64_t>(ws.capacity, total - base);
    P.chunk_base = base;
    RET_CUDA(runChunk(stream, A, S, P, st, Q, counters, count, p.max_depth, d_film, G));
  }
  unsigned long long cnt[C_COUNT];
  RET_CUDA(cudaMemcpyAsync(cnt, counters, sizeof cnt, cudaMemcpyDeviceToHost, stream));
  RET_CUDA(cudaStreamSynchronize(stream));
  res.rays_closest = cnt[C_CLOSEST];
  res.rays_any = cnt[C_ANY];
  res.nonfinite = cnt[C_NONFINITE];
  res.degenerate = cnt[C_DEGENERATE];
  res.path_samples = total;
  return BLING_OK;
}

// ------------------------------------------------------------------ no-allocation pass
// Path state for bling_render_pass_noalloc, in one file-scope device array:
// the wavefront of one pass of at most kNoAllocSlots path samples (slots,
// queues and counters, laid out by carve()).  Every GPU that loads the library
// holds it (about 35 MiB) until the process exits.  All calls share the array;
// the counters are cleared at the start of every call and the path state is
// written before it is read.  Two calls whose work overlaps on the GPU
// (different streams or contexts on one device) race on it.
constexpr size_t kNoAllocSlots = size_t(1) << 16;
constexpr size_t kNoAllocBytes = kCounterBytes + (kSlotWords + kQueueWords) * 4 * kNoAllocSlots;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {
constexpr int kMaxDevices = 64;
unsigned char* g_noalloc_ptr[kMaxDevices] = {nullptr};
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
  if (!g_noalloc_ptr[device]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
      err = std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e);
      return BLING_ERR_CUDA;
    }
    g_noalloc_ptr[device] = (unsigned char*)ptr;
  }
  RET_CUDA(ensureConstants(device));
  PassParams P;
  int rc = passParams(p, pass, fw, fh, P, err);
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
  float tbl[256];
  filterTableHost(p.filter_kind, p.filter_params, P.fw, P.fh, tbl);
  RET_CUDA(cudaMemcpyToSymbolAsync(c_filter, tbl, sizeof tbl, 0, cudaMemcpyHostToDevice, stream));
  Slots st;
  Queues Q;
  unsigned long long* counters;
  carve(g_noalloc_ptr[device], kNoAllocSlots, st, Q, counters);
  RET_CUDA(cudaMemsetAsync(counters, 0, C_COUNT * sizeof(unsigned long long), stream));
  int sms = 0;
  RET_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  Grids G = grids(device, sms);
  P.chunk_base = 0;
  RET_CUDA(runChunk(stream, A, S, P, st, Q, counters, (int64_t)total, p.max_depth, d_film, G));
  unsigned long long cnt[C_COUNT];
  RET_CUDA(cudaMemcpyAsync(cnt, counters, sizeof cnt, cudaMemcpyDeviceToHost, stream));
  RET_CUDA(cudaStreamSynchronize(stream));
  res.rays_closest = cnt[C_CLOSEST];
  res.rays_any = cnt[C_ANY];
  res.nonfinite = cnt[C_NONFINITE];
  res.degenerate = cnt[C_DEGENERATE];
  res.path_samples = total;
  return BLING_OK;
}

}  // namespace bgpu
