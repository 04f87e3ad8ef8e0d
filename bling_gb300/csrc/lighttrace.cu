// Wavefront light tracer on the GPU.
//
// One pass of the reference's light tracer (Renderer/LightTracer.hs:37-110):
// `photons` paths leave the scene's lights (sampleLightRay, Scene.hs:121-135;
// sample', Light.hs:166-213) and bounce by adjoint BSDF sampling
// (sampleAdjBsdf, Reflection.hs:272-316); every vertex is connected to the
// camera (connectCam / sampleCam, LightTracer.hs:57-71, Camera.hs:90-100) and,
// when the connection is unoccluded, splatted into the film's splat image
// (splatSample, Image.hs:201-221).  Russian roulette continues a path with
// probability 0.8 after its fourth vertex; the reference has no depth limit.
//
// Photons live in slots that never move; queues of slot indices carry the live
// photons from launch to launch.  Each bounce is three launches:
//
//   k_lt_trace   closest hit of the live photons' rays (scIntersect)
//   k_lt_vertex  the BSDF at the hit, the camera connection (queued as a
//                shadow ray with its splat) and the continuation sample
//   k_lt_shadow  any hit of the camera connections; unoccluded ones add their
//                XYZ to the splat image (atomics: the order of the additions
//                into a pixel varies, their terms do not)
//
// Random numbers come from the counter-based generator shared with the CPU
// oracle, keyed by (seed, pass, photon): dimension 0 picks the light, 1-2 the
// point on it, 3-4 the direction; vertex d draws 5+4d (BSDF component), 6+4d
// and 7+4d (direction) and 8+4d (roulette).
#include <algorithm>
#include <cstring>

#include "lighttrace.h"
#include "photon.cuh"

namespace bgpu {

namespace {

enum : int {
  L_LIVE0 = 0, L_LIVE1 = 1, L_CLOSEST = 2, L_ANY = 3, L_NONFINITE = 4, L_NEXT_TRACE = 5,
  L_SHADOW = 6, L_NEXT_SHADOW = 7, L_DEGENERATE = 8, L_SPLATS = 9, L_COUNT = 16
};

// per photon: li 16, ray 8, wi 4, hit 4, shadow ray 8, splat 4 words; 3 queues
constexpr size_t kLtSlotWords = 16 + 8 + 4 + 4 + 8 + 4;
constexpr size_t kLtQueueWords = 3;
constexpr size_t kLtCounterBytes = 256;

struct LtSlots {
  float* li;       // 16 per photon: the photon's power (li of nextVertex)
  float* ray;      // 8 per photon: the ray to trace next
  float4* wi;      // per photon: direction back along the path (x, y, z, unused)
  float4* hit;     // per photon: t, primitive ID (int bits; -1 none), b1, b2
  float* sray;     // 8 per photon: the camera connection o, d, tmin, tmax
  float4* splat;   // per photon: pixel index (int bits; -1 non-finite), X, Y, Z
  int32_t* live[2];
  int32_t* shadow;
};

struct LtParams {
  uint64_t seed, pass, chunk_base;
  int width, height;
  int max_depth;
  V3 wc;     // bounding sphere of the scene (boundingSphere, AABB.hs:62-66)
  float wr;
};

size_t ltBytes(size_t cap) { return kLtCounterBytes + (kLtSlotWords + kLtQueueWords) * 4 * cap; }

void ltCarve(unsigned char* base, size_t cap, LtSlots& st, unsigned long long*& counters) {
  counters = (unsigned long long*)base;
  float* w = (float*)(base + kLtCounterBytes);
  auto take = [&](size_t words) {
    float* p = w;
    w += words * cap;
    return p;
  };
  st.li = take(16);
  st.ray = take(8);
  st.wi = reinterpret_cast<float4*>(take(4));
  st.hit = reinterpret_cast<float4*>(take(4));
  st.sray = take(8);
  st.splat = reinterpret_cast<float4*>(take(4));
  st.live[0] = (int32_t*)take(1);
  st.live[1] = (int32_t*)take(1);
  st.shadow = (int32_t*)take(1);
}

// ------------------------------------------------------------------ kernels
// oneRay (LightTracer.hs:46-55): the first ray and power of photons
// [chunk_base, chunk_base + count)
__global__ void __launch_bounds__(128) k_lt_emit(DevAccel A, DevShading S, LtParams P, LtSlots st,
                                                 int64_t count, unsigned long long* counters) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t nround = (count + stride - 1) / stride * stride;
  int lc = S.n_lights;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nround; i += stride) {
    bool live = false;
    if (i < count && lc > 0) {
      uint64_t g = P.chunk_base + (uint64_t)i;
      uint64_t key = photonKey(P.seed, P.pass, g);
      uint32_t n = (uint32_t)g;
      float ul = randF(key, n, 0);
      float uo1 = randF(key, n, 1), uo2 = randF(key, n, 2);
      float ud1 = randF(key, n, 3), ud2 = randF(key, n, 4);
      int ln = lc == 1 ? 0 : min((int)floorf(ul * (float)lc), lc - 1);
      Spec le;
      Ray ray;
      V3 nl;
      float pdf;
      lightEmit(A, S, S.lights[ln], P.wc, P.wr, uo1, uo2, ud1, ud2, le, ray, nl, pdf);
      if (lc != 1) pdf = pdf / (float)lc;
      V3 wo = normalize(ray.d);
      Spec li = sScale(le, absDot(nl, wo) / pdf);
      live = pdf > 0 && !isBlack(li);
      if (live) {
        storeBands(st.li, (int)i, li);
        storeRay(st.ray, (int)i, ray);
        st.wi[i] = make_float4(-wo.x, -wo.y, -wo.z, 0.0f);
      }
    }
    queueAppend(live, (int)i, st.live[0], counters + L_LIVE0);
  }
}

// zeroes the per-bounce counters and the next live queue's size
__global__ void k_lt_reset(unsigned long long* counters, int next_live) {
  int t = threadIdx.x;
  if (t == 0) counters[next_live] = 0;
  if (t == 1) counters[L_NEXT_TRACE] = 0;
  if (t == 2) counters[L_SHADOW] = 0;
  if (t == 3) counters[L_NEXT_SHADOW] = 0;
}

template <int LAYOUT>
__global__ void __launch_bounds__(128, 8) k_lt_trace(DevAccel A, LtSlots st, int in,
                                                      unsigned long long* __restrict__ counters) {
  const int32_t* __restrict__ queue = st.live[in];
  int64_t n = (int64_t)counters[L_LIVE0 + in];
  traceWarpPersistent<false, LAYOUT, false>(
      A, n, counters + L_NEXT_TRACE, [&](int64_t q) { return loadRay7(st.ray, queue[q]); },
      [&](int64_t q, const RayQueryResult& res) {
        st.hit[queue[q]] = hitRecord(res.hit, res.t, res.prim, res.b1, res.b2);
      });
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(counters + L_CLOSEST, (unsigned long long)n);
}

// nextVertex (LightTracer.hs:73-110) of every live photon at vertex `depth`,
// with its camera connection (connectCam, LightTracer.hs:57-71).  TEX: the
// scene has textured materials.
template <bool TEX>
__global__ void __launch_bounds__(128, 4) k_lt_vertex(DevAccel A, DevShading S, LtParams P,
                                                      LtSlots st, int depth, int in,
                                                      unsigned long long* __restrict__ counters) {
  const int32_t* __restrict__ qin = st.live[in];
  int64_t n = (int64_t)counters[L_LIVE0 + in];
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t nround = (n + stride - 1) / stride * stride;
  const bling_camera_desc& cam = S.camera;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nround; q += stride) {
    bool shadow = false, cont = false;
    int s = 0;
    if (q < n) {
      s = qin[q];
      const float4 hit = st.hit[s];
      int prim = __float_as_int(hit.y);
      Spec li = loadBands(st.li, s);
      if (prim == kDegenerateRay) {
        // a NaN ray: every later splat of the reference's photon is NaN and dropped
        atomicAdd(counters + L_DEGENERATE, 1ull);
      } else if (prim >= 0 && !isBlack(li)) {
        uint64_t g = P.chunk_base + (uint64_t)s;
        uint64_t key = photonKey(P.seed, P.pass, g);
        uint32_t rn = (uint32_t)g;
        uint32_t dim = 5 + 4 * (uint32_t)depth;
        float ubc = randF(key, rn, dim), ubd1 = randF(key, rn, dim + 1),
              ubd2 = randF(key, rn, dim + 2);
        float pcont = depth > 3 ? 0.8f : 1.0f;
        Ray ray = loadRay7(st.ray, s);
        HitGeom hg = hitGeometry(A, S, ray, prim, hit.x, hit.z, hit.w);
        DMaterial tm;  // a textured material, resolved at this hit
        const DMaterial* mat = S.materials + hg.material;
        if constexpr (TEX) mat = hitMaterial(A, S, ray, prim, hit.x, hit.z, hit.w, hg, tm);
        Bsdf bsdf = materialBsdf(*mat, hg.n, hg.sp, hg.sn, hg.sdpdu);
        float4 w4 = st.wi[s];
        V3 wi{w4.x, w4.y, w4.z};
        V3 p = bsdf.p;
        BsdfSample bs = sampleBsdf<true>(bsdf, wi, ubc, ubd1, ubd2);  // sampleAdjBsdf
        // connectCam: sampleCam of the projective camera (Camera.hs:95-100)
        V3 pRas = transPoint(cam.w2r, p);
        V3 pCam = transPoint(cam.c2w, V3{0, 0, 0});
        float cost = fabsf(normalize(transPoint(cam.r2c, pRas)).z);
        float cost3 = cost * cost * cost;
        float cPdf = cam.pixel_area * cost3;
        V3 dCam = pCam - p;
        V3 we = normalize(dCam);
        Spec f = evalBsdf<true>(bsdf, wi, we);
        if (!isBlack(f) && cPdf != 0) {
          float dCam2 = sqLen(dCam);
          Spec lr = sScale(li * f, 1.0f / (cPdf * dCam2));
          float px = pRas.x, py = pRas.y;
          // splatSample drops splats outside the image; they need no visibility
          if (px >= 0.0f && px < (float)P.width && py >= 0.0f && py < (float)P.height) {
            bool bad = false;
#pragma unroll
            for (int i = 0; i < 16; i++) bad = bad || isnan(lr.v[i]) || isinf(lr.v[i]);
            float x = 0, y = 0, z = 0;
#pragma unroll
            for (int i = 0; i < 16; i++) {
              x = x + c_cieX[i] * lr.v[i];
              y = y + c_cieY[i] * lr.v[i];
              z = z + c_cieZ[i] * lr.v[i];
            }
            int pix = (int)floorf(py) * P.width + (int)floorf(px);
            st.splat[s] = make_float4(__int_as_float(bad ? -1 : pix), x / c_cieYSum,
                                      y / c_cieYSum, z / c_cieYSum);
            storeRay(st.sray, s, Ray{p, we, hg.eps, sqrtf(dCam2)});
            shadow = true;
          }
        }
        if (!isBlack(bs.f) && bs.pdf != 0 && !(randF(key, rn, dim + 3) > pcont) &&
            !(P.max_depth > 0 && depth + 1 >= P.max_depth)) {
          storeBands(st.li, s, sScale(li * bs.f, 1.0f / pcont));
          storeRay(st.ray, s, Ray{p, bs.wi, hg.eps, INFINITY});
          st.wi[s] = make_float4(-bs.wi.x, -bs.wi.y, -bs.wi.z, 0.0f);
          cont = true;
        }
      }
    }
    queueAppend(shadow, s, st.shadow, counters + L_SHADOW);
    queueAppend(cont, s, st.live[1 - in], counters + L_LIVE0 + (1 - in));
  }
}

// occluded (Scene.hs:45-47) for the camera connections; the visible ones
// are splatted
template <int LAYOUT>
__global__ void __launch_bounds__(128, 8) k_lt_shadow(DevAccel A, LtSlots st,
                                                       float* __restrict__ splat_xyz,
                                                       unsigned long long* __restrict__ counters) {
  const int32_t* __restrict__ queue = st.shadow;
  int64_t n = (int64_t)counters[L_SHADOW];
  traceWarpPersistent<true, LAYOUT, false>(
      A, n, counters + L_NEXT_SHADOW,
      [&](int64_t q) {
        const float4* p = reinterpret_cast<const float4*>(st.sray + 8 * (size_t)queue[q]);
        float4 a = p[0], b = p[1];
        return Ray{V3{a.x, a.y, a.z}, V3{a.w, b.x, b.y}, b.z, b.w};
      },
      [&](int64_t q, const RayQueryResult& res) {
        if (res.prim == kDegenerateRay) atomicAdd(counters + L_DEGENERATE, 1ull);
        if (res.hit) return;
        float4 sp = st.splat[queue[q]];
        int pix = __float_as_int(sp.x);
        if (pix < 0) {
          atomicAdd(counters + L_NONFINITE, 1ull);
          return;
        }
        float* o = splat_xyz + 3 * (size_t)pix;
        atomicAdd(o, sp.y);
        atomicAdd(o + 1, sp.z);
        atomicAdd(o + 2, sp.w);
        atomicAdd(counters + L_SPLATS, 1ull);
      });
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(counters + L_ANY, (unsigned long long)n);
}

template <class K>
unsigned residentGrid(K kernel, int sms) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0);
  return (unsigned)(std::max(1, sms) * std::max(1, per_sm));
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

void light_workspace_free(LightWorkspace& ws) {
  cudaFree(ws.buffer);
  ws = LightWorkspace{};
}

int light_pass(cudaStream_t stream, const DevAccel& A, const DevShading& S, const LightPassArgs& a,
               float* d_splat, LightWorkspace& ws, LightPassResult& res, std::string& err) {
  int device = 0;
  RET_CUDA(cudaGetDevice(&device));
  RET_CUDA(loadCieConstants(device));
  res = LightPassResult{};
  if (a.photons <= 0) return BLING_OK;
  // a multiple of 64 photons keeps every per-photon array 16-byte aligned
  size_t cap = (size_t)std::min<int64_t>(a.photons, int64_t(1) << 22);
  cap = (std::max<size_t>(cap, 1024) + 63) / 64 * 64;
  if (ws.capacity < cap || !ws.buffer) {
    light_workspace_free(ws);
    RET_CUDA(cudaMalloc(&ws.buffer, ltBytes(cap)));
    ws.capacity = cap;
  }
  LtSlots st;
  unsigned long long* counters;
  ltCarve((unsigned char*)ws.buffer, ws.capacity, st, counters);
  RET_CUDA(cudaMemsetAsync(counters, 0, L_COUNT * sizeof(unsigned long long), stream));
  LtParams P;
  P.seed = a.seed;
  P.pass = a.pass;
  P.width = a.width;
  P.height = a.height;
  P.max_depth = a.max_depth;
  P.wc = V3{a.wc[0], a.wc[1], a.wc[2]};
  P.wr = a.wr;
  int sms = 0;
  RET_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int block = 128;
  unsigned g_trace = withLayout(A.wide, [&](auto L) {
    return residentGrid(k_lt_trace<decltype(L)::value>, sms);
  });
  unsigned g_shadow = withLayout(A.wide, [&](auto L) {
    return residentGrid(k_lt_shadow<decltype(L)::value>, sms);
  });
  unsigned g_vertex = residentGrid(k_lt_vertex<false>, sms);
  unsigned g_emit = (unsigned)std::max(1, sms * 8);
  for (int64_t base = 0; base < a.photons; base += (int64_t)ws.capacity) {
    int64_t count = std::min<int64_t>((int64_t)ws.capacity, a.photons - base);
    P.chunk_base = (uint64_t)base;
    unsigned cap_blocks = (unsigned)std::max<int64_t>(1, (count + block - 1) / block);
    k_lt_reset<<<1, 32, 0, stream>>>(counters, L_LIVE0);
    k_lt_emit<<<std::min(g_emit, cap_blocks), block, 0, stream>>>(A, S, P, st, count, counters);
    RET_CUDA(cudaGetLastError());
    // The reference has no depth limit: bounces run until no photon is left.
    // The live count is read back every few bounces once the first ones are
    // done (launches on an empty queue cost a few microseconds).
    for (int depth = 0;; depth++) {
      int in = depth & 1;
      k_lt_reset<<<1, 32, 0, stream>>>(counters, L_LIVE0 + (1 - in));
      unsigned gt = std::min(g_trace, cap_blocks), gs = std::min(g_shadow, cap_blocks),
               gv = std::min(g_vertex, cap_blocks);
      withLayout(A.wide, [&](auto L) {
        k_lt_trace<decltype(L)::value><<<gt, block, 0, stream>>>(A, st, in, counters);
      });
      if (S.textured)
        k_lt_vertex<true><<<gv, block, 0, stream>>>(A, S, P, st, depth, in, counters);
      else
        k_lt_vertex<false><<<gv, block, 0, stream>>>(A, S, P, st, depth, in, counters);
      withLayout(A.wide, [&](auto L) {
        k_lt_shadow<decltype(L)::value><<<gs, block, 0, stream>>>(A, st, d_splat, counters);
      });
      RET_CUDA(cudaGetLastError());
      if (depth >= 7 && (depth & 3) == 3) {
        unsigned long long live = 0;
        RET_CUDA(cudaMemcpyAsync(&live, counters + L_LIVE0 + (1 - in), sizeof live,
                                 cudaMemcpyDeviceToHost, stream));
        RET_CUDA(cudaStreamSynchronize(stream));
        if (live == 0) break;
      }
      if (a.max_depth > 0 && depth + 1 >= a.max_depth) break;
    }
  }
  unsigned long long cnt[L_COUNT];
  RET_CUDA(cudaMemcpyAsync(cnt, counters, sizeof cnt, cudaMemcpyDeviceToHost, stream));
  RET_CUDA(cudaStreamSynchronize(stream));
  res.rays_closest = cnt[L_CLOSEST];
  res.rays_any = cnt[L_ANY];
  res.splats = cnt[L_SPLATS];
  res.nonfinite = cnt[L_NONFINITE];
  res.degenerate = cnt[L_DEGENERATE];
  res.photons = (uint64_t)a.photons;
  return BLING_OK;
}

}  // namespace bgpu
