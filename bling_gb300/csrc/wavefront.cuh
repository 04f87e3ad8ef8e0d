// Wavefront building blocks shared by the per-pass integrator (integrator.cu)
// and the batched job engine (batch.cu): the SoA path slots, queue appends,
// camera rays, and the two halves of one path vertex (nextVertex,
// Integrator/Path.hs:49-87) around its deferred shadow and MIS rays.
//
// Paths live in slots (throughput and radiance as 16-band spectra,
// band-major) and never move; queues of slot indices carry the live paths from
// stage to stage.  Arithmetic keeps the reference's operation order
// (-fmad=false); random numbers come from the counter-based generator shared
// with the CPU oracle, keyed by (seed, pass, pixel, sample index), so a path's
// result does not depend on the slot or the launch that carries it.
#pragma once
#include "integrator_device.cuh"

namespace bgpu {

// VF_LE: the vertex saw emission (a specular path hit an area light); its
// spectrum is in intl, which is neither written nor read otherwise
enum : int { VF_SHADOW = 1, VF_MIS = 2, VF_CONT = 4, VF_LE = 8 };

struct Slots {
  size_t cap;
  float* T;          // 16 per path
  float* L;          // 16 per path
  float* ray;        // 8 per path: o, d, tmin (sign bit: the previous bounce was specular), tmax
  float4* hit;       // per path: t, primitive ID (int bits; -1 none), b1, b2
  // the current vertex, deferred until its shadow and MIS rays are traced
  float* intl;       // 16 per path: emission seen on a specular path
  float* ls;         // 16 per path: light-sample term before visibility
  float* bsf;        // 16 per path: MIS BSDF sample throughput
  float* fc;         // 16 per path: continuation BSDF sample throughput
  float* bsw;        // cap: MIS weight of the BSDF sample
  float* invpc;      // cap: 1 / continuation probability
  int32_t* vflags;   // cap: VF_* | light index << 8
  float* sray;       // 8 per path: shadow ray o, d, tmin, tmax
  int32_t* svis;     // cap: shadow ray unoccluded
  float* mray;       // 8 per path: MIS ray o, d, tmin, tmax
  float4* mhit;      // per path: the MIS ray's hit, as hit
};

struct Queues {
  int32_t* live[2];  // paths to trace this bounce / next bounce
  int32_t* shadow;   // 2 cap entries: shadow rays and MIS rays (occlusionSlot)
  int32_t* resolve;
  int32_t* sorted;   // the live paths in shading-class order
  int32_t* cls;      // shading class per live queue entry
};

// counters (unsigned long long): queue sizes and statistics
enum : int {
  C_LIVE0 = 0, C_LIVE1 = 1, C_CLOSEST = 2, C_ANY = 3, C_NONFINITE = 4, C_NEXT_TRACE = 5,
  C_SHADOW = 6, C_RESOLVE = 8, C_NEXT_SHADOW = 9, C_DEGENERATE = 11,
  C_FIRST_NONFINITE = 12,  // ~g of the pass's lowest dropped sample g (0: none), by atomicMax
  C_COUNT = 16
};

constexpr size_t kSlotWords = 16 * 6 + 8 + 4 + 3 + 8 + 1 + 8 + 4;  // per slot, 4-byte words
constexpr size_t kQueueWords = 7;  // the shadow queue takes two
// counters: C_COUNT 8-byte counters, then the shading-class counts and
// cursors (kShadeClasses 4-byte entries each, 16 reserved)
constexpr size_t kCounterBytes = 256;
constexpr int kClassCountsAt = C_COUNT * 2;  // in 4-byte words

// carves the slot arrays (kSlotWords per slot) from w, advancing it
inline void carveSlots(float*& w, size_t cap, Slots& st) {
  auto take = [&](size_t words) {
    float* p = w;
    w += words * cap;
    return p;
  };
  st.cap = cap;
  st.T = take(16);
  st.L = take(16);
  st.ray = take(8);
  st.hit = reinterpret_cast<float4*>(take(4));
  st.intl = take(16);
  st.ls = take(16);
  st.bsf = take(16);
  st.fc = take(16);
  st.bsw = take(1);
  st.invpc = take(1);
  st.vflags = (int32_t*)take(1);
  st.sray = take(8);
  st.svis = (int32_t*)take(1);
  st.mray = take(8);
  st.mhit = reinterpret_cast<float4*>(take(4));
}

// sample index g of a pass -> pixel and sample number (pixel-major, like the
// tile loop of prender, Rendering.hs:127-140)
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
// the camera sample (runSample, Sampling.hs:101-132): stratified pixel
// positions and shuffled stratified lens positions, or for the Random sampler
// four independent uniforms
__device__ __forceinline__ void pixelSample(const PassParams& P, const Sampler& s, int ix, int iy,
                                            float& sx, float& sy, float& lu, float& lv) {
  float ox, oy;
  if (P.random) {
    ox = randF(s.key, s.n, DIM_PIX_U);
    oy = randF(s.key, s.n, DIM_PIX_V);
    lu = randF(s.key, s.n, DIM_LENS_U);
    lv = randF(s.key, s.n, DIM_LENS_V);
  } else {
    strat2D(s, s.n, DIM_PIX_U, DIM_PIX_V, ox, oy);
    uint32_t N = (uint32_t)P.spp;
    uint32_t lp = permute(s.n, N, randU32(s.key, 0xffffffffu, DIM_LENS_PERM));
    strat2D(s, lp, DIM_LENS_U, DIM_LENS_V, lu, lv);
  }
  sx = (float)ix + ox;
  sy = (float)iy + oy;
}

// Per-path records.  A bounce visits its paths in shading-class order, so
// the lanes of a warp touch scattered paths: spectra are stored per path
// (16 consecutive floats, 64 bytes) and rays as 8 floats (o, d, tmin, tmax),
// so that a lane's loads fill whole 32-byte sectors instead of one float
// per sector.
__device__ __forceinline__ Spec loadBands(const float* base, int s) {
  const float4* p = reinterpret_cast<const float4*>(base + 16 * (size_t)s);
  Spec v;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    float4 q = p[k];
    v.v[4 * k] = q.x;
    v.v[4 * k + 1] = q.y;
    v.v[4 * k + 2] = q.z;
    v.v[4 * k + 3] = q.w;
  }
  return v;
}
__device__ __forceinline__ void storeBands(float* base, int s, const Spec& v) {
  float4* p = reinterpret_cast<float4*>(base + 16 * (size_t)s);
#pragma unroll
  for (int k = 0; k < 4; k++)
    p[k] = make_float4(v.v[4 * k], v.v[4 * k + 1], v.v[4 * k + 2], v.v[4 * k + 3]);
}
// a ray record: the sign bit of tmin may carry a flag (loadRay7 drops it)
__device__ __forceinline__ void storeRay(float* base, int s, const Ray& r) {
  float4* p = reinterpret_cast<float4*>(base + 8 * (size_t)s);
  p[0] = make_float4(r.o.x, r.o.y, r.o.z, r.d.x);
  p[1] = make_float4(r.d.y, r.d.z, r.tmin, r.tmax);
}
__device__ __forceinline__ void copyRay(const float* from, int q, float* to, int p) {
  const float4* a = reinterpret_cast<const float4*>(from + 8 * (size_t)q);
  float4* b = reinterpret_cast<float4*>(to + 8 * (size_t)p);
  b[0] = a[0];
  b[1] = a[1];
}
// a hit record: t, the primitive ID as int bits (-1: no hit), barycentrics
__device__ __forceinline__ float4 hitRecord(bool hit, float t, int prim, float b1, float b2) {
  return make_float4(t, __int_as_float(hit ? prim : -1), b1, b2);
}
__device__ __forceinline__ int hitPrim(const float4* rec, int s) {
  return __float_as_int(reinterpret_cast<const float*>(rec + s)[1]);
}
__device__ __forceinline__ float rayTminBits(const float* base, int s) {
  return base[8 * (size_t)s + 6];
}
// a closest-hit ray (tmax = infinity, tmin without its flag)
__device__ __forceinline__ Ray loadRay7(const float* base, int s) {
  const float4* p = reinterpret_cast<const float4*>(base + 8 * (size_t)s);
  float4 a = p[0], b = p[1];
  return Ray{V3{a.x, a.y, a.z}, V3{a.w, b.x, b.y}, fabsf(b.z), INFINITY};
}
// a whole ray record (o, d, tmin, tmax)
__device__ __forceinline__ Ray loadRay8(const float* base, int s) {
  const float4* p = reinterpret_cast<const float4*>(base + 8 * (size_t)s);
  float4 a = p[0], b = p[1];
  return Ray{V3{a.x, a.y, a.z}, V3{a.w, b.x, b.y}, b.z, b.w};
}
__device__ __forceinline__ Ray loadShadowRay(const Slots& st, int s) { return loadRay8(st.sray, s); }

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

// ---- shading classes.  Before shading, the live paths of a bounce are
// reordered by what their vertex runs: 0 for a miss or a degenerate ray (the
// path ends), else 1 + the hit material's kind + kMaterialKinds for an analytic shape
// (triangles and shapes build their geometry differently).  Lanes of a warp
// then run one BSDF's and one geometry's code instead of all of them in turn.
// The order within a class is the queue's order, up to the interleaving of
// warps.
constexpr int kMaterialKinds = 7;  // BLING_MAT_MATTE .. BLING_MAT_TRANS_MATTE; substrate sorts with plastic
constexpr int kShadeClasses = 1 + 2 * kMaterialKinds;
static_assert(kShadeClasses <= 16, "class counts and cursors hold 16 entries each");

__device__ __forceinline__ int shadeClass(const DevAccel& A, const DevShading& S, int prim) {
  if (prim < 0) return 0;
  int2 info = __ldg(S.prim_info + prim);
  int mi, shape = 0;
  if (info.x >= 0) {
    mi = S.meshes[info.x].material;
  } else {
    mi = A.shapes[~info.x].material;
    shape = 1;
  }
  int kind = S.materials[mi].kind;
  if (kind == BLING_MAT_SUBSTRATE) kind = BLING_MAT_PLASTIC;  // both glossy, one class
  if (kind == BLING_MAT_BLACKBODY) kind = BLING_MAT_MATTE;    // no BxDF: the path ends
  return 1 + kind + kMaterialKinds * shape;
}

// counts a warp's entries per class (one atomic per class present); every
// lane of the warp calls it, c < 0 for lanes without an entry
__device__ __forceinline__ void classCount(int c, unsigned* __restrict__ counts) {
  unsigned grp = __match_any_sync(0xffffffffu, c);
  if (c >= 0 && (threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(counts + c, (unsigned)__popc(grp));
}

// the entry's position in the class-sorted order: the class's offset (off,
// exclusive prefix of the counts) plus its rank; every lane calls it
__device__ __forceinline__ int classSlot(int c, const unsigned* off, unsigned* __restrict__ cursor) {
  const int lane = threadIdx.x & 31;
  unsigned grp = __match_any_sync(0xffffffffu, c);
  int leader = __ffs(grp) - 1;
  unsigned base = 0;
  if (c >= 0 && lane == leader) base = atomicAdd(cursor + c, (unsigned)__popc(grp));
  base = __shfl_sync(0xffffffffu, base, leader);
  return c >= 0 ? (int)(off[c] + base + __popc(grp & ((1u << lane) - 1))) : -1;
}

// exclusive prefix of the class counts into shared memory (block-wide)
__device__ __forceinline__ void classOffsets(const unsigned* __restrict__ counts, unsigned* off) {
  if (threadIdx.x == 0) {
    unsigned run = 0;
    for (int c = 0; c < kShadeClasses; c++) {
      off[c] = run;
      run += counts[c];
    }
  }
  __syncthreads();
}

// intLe (Primitive.hs:68-76) + lEmit (Light.hs:85-96)
__device__ __forceinline__ Spec intLe(const DevShading& S, const HitGeom& g, V3 wo) {
  if (g.light_id < 0) return sConst(0);
  return dot(g.n, wo) > 0 ? sLoad(S.shape_emission + 16 * g.shape) : sConst(0);
}

// camera ray of sample g (fireRay, Camera.hs:49-68)
__device__ __forceinline__ Ray cameraRay(const PassParams& P, const bling_camera_desc& cam,
                                         uint64_t g) {
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
  return transRay(cam.c2w, ray);
}

// the film splat of sample g (the raster position is recomputed from the
// sampler); false when the sample is dropped as NaN/Inf (counted in
// *nonfinite)
template <class Filter>
__device__ __forceinline__ bool splatSampleAt(float* film, const PassParams& P, uint64_t g,
                                              const Spec& L, unsigned long long* nonfinite,
                                              Filter filt) {
  int ix, iy;
  uint32_t sn;
  decodeSample(P, g, ix, iy, sn);
  Sampler smp = mkSampler(P, ix, iy, sn);
  float sx, sy, lu, lv;
  pixelSample(P, smp, ix, iy, sx, sy, lu, lv);
  return filmAddT(film, P, ix, iy, sx, sy, L, nonfinite, filt);
}
// splatSampleAt with the path integrator's counters: a dropped sample counts
// in counters[C_NONFINITE] and the lowest such g is kept in
// counters[C_FIRST_NONFINITE]
template <class Filter>
__device__ __forceinline__ void splatSample(float* film, const PassParams& P, uint64_t g,
                                            const Spec& L, unsigned long long* counters,
                                            Filter filt) {
  if (!splatSampleAt(film, P, g, L, counters + C_NONFINITE, filt))
    atomicMax(counters + C_FIRST_NONFINITE, ~(unsigned long long)g);
}

// the pass constants of render parameters (imageWindow', Image.hs:170-176;
// Path.hs:34-36), integrator.cu
int integrator_pass_params(const bling_render_params& p, uint64_t pass, int fw, int fh,
                           PassParams& P, std::string& err);

struct VertexOut {
  bool shadow, mis, resolve;
};

// Entries of the shadow queue: a slot s (its shadow ray, visibility into
// svis), or ~s for the slot's MIS ray.  The closest-hit query of
// sampleBsdfMis (Scene.hs:71-82) only matters through whether its answer is
// the sampled light, or, for a light that is not an area light, whether
// there is any answer, so each MIS ray becomes an occlusion query:
//  * toward an area light whose shape the ray meets at t_L (the shape's own
//    Shape.intersect, as the traversal computes it): is there a primitive
//    that a closest-hit query would rank before it, i.e. one hit at t < t_L
//    or at t_L with a larger primitive ID (nearest', Primitive.hs:29-43)?
//    mhit holds the light's hit (t_L, its primitive) until an occluder
//    replaces it;
//  * otherwise: is there any hit at all?  mhit holds a miss until a hit
//    replaces it.
// The shadow kernel walks both with the any-hit traversal in MIXED mode: an
// MIS entry's shapes answer by Shape.intersect, as the closest-hit query
// would, a shadow ray's by Shape.intersects; the primitive an area light
// entry ranks against comes from its mhit record.
__device__ __forceinline__ int occlusionSlot(int e) { return e >= 0 ? e : ~e; }
__device__ __forceinline__ Ray loadOcclusionRay(const Slots& st, int e, bool& by_intersect,
                                                int& rank_prim) {
  by_intersect = e < 0;
  if (e >= 0) {
    rank_prim = -1;
    return loadShadowRay(st, e);
  }
  rank_prim = __float_as_int(st.mhit[~e].y);  // the light's primitive, or -1
  return loadRay8(st.mray, ~e);
}
__device__ __forceinline__ void storeOcclusion(const Slots& st, int e, const RayQueryResult& res,
                                               unsigned long long* degenerate) {
  if (e >= 0) {
    st.svis[e] = res.hit ? 0 : 1;
    if (res.prim == kDegenerateRay) atomicAdd(degenerate, 1ull);
  } else if (res.hit) {
    st.mhit[~e] = hitRecord(true, res.t, res.prim, res.b1, res.b2);
  }
}

// First half of one vertex of the path in slot s at bounce `depth`
// (Path.hs:49-87): emission on specular paths, the BSDF, one light sample
// and one BSDF sample for MIS (sampleOneLight/estimateDirect,
// Scene.hs:61-118), Russian roulette and the continuation sample.  Stores
// the deferred terms in the slot and says which rays to trace; a path that
// ends here is handed to finish(L).  TEX: the scene has textured materials
// (the variant without them makes no out-of-line call).
template <bool TEX, class Finish>
__device__ __forceinline__ VertexOut shadeVertex(const DevAccel& A, const DevShading& S,
                                                 const PassParams& P, const Slots& st, int s,
                                                 uint64_t g, int depth,
                                                 unsigned long long* counters, Finish finish) {
  VertexOut out{false, false, false};
  int ix, iy;
  uint32_t sn;
  decodeSample(P, g, ix, iy, sn);
  Sampler smp = mkSampler(P, ix, iy, sn);
  size_t c = st.cap;
  Ray ray = loadRay7(st.ray, s);
  bool specular = depth == 0 || signbit(rayTminBits(st.ray, s));
  const float4 hit = st.hit[s];
  int prim = __float_as_int(hit.y);
  if (prim == kDegenerateRay) {
    // a NaN ray: the reference's sample ends NaN and is dropped by the film
    atomicAdd(counters + C_DEGENERATE, 1ull);
    finish(sConst(NAN));
    return out;
  }
  if (prim < 0 || depth == P.max_depth) {
    Spec Lr = loadBands(st.L, s);
    if (prim < 0 && specular) {  // nothing hit after a specular bounce: l + t * sum le
      Spec sum = sConst(0);
      for (int k = 0; k < S.n_lights; k++) sum = sum + lightLe(S.lights[k], ray.d);
      Lr = Lr + loadBands(st.T, s) * sum;
    }
    finish(Lr);
    return out;
  }
  float thit = hit.x, b1 = hit.z, b2 = hit.w;
  HitGeom gm = hitGeometry(A, S, ray, prim, thit, b1, b2);
  V3 rd = ray.d;
  int flags = 0;
  if (specular && gm.light_id >= 0) {
    storeBands(st.intl, s, intLe(S, gm, rd));
    flags |= VF_LE;
  }
  DMaterial tm;  // a textured material, resolved at this hit
  const DMaterial* mat = S.materials + gm.material;
  if constexpr (TEX) mat = hitMaterial(A, S, ray, prim, thit, b1, b2, gm, tm);
  V3 wo = -rd;
  float lNumU = rnd1(smp, 1 + 4 * depth);
  float ld1, ld2;
  rnd2(smp, 1 + 3 * depth, ld1, ld2);
  float lBsdfCompU = rnd1(smp, 2 + 4 * depth);
  float lb1, lb2;
  rnd2(smp, 2 + 3 * depth, lb1, lb2);
  Bsdf bsdf = materialBsdf(*mat, gm.n, gm.sp, gm.sn, gm.sdpdu);
  V3 nn = bsdf.cs.n, p = bsdf.p;
  float eps = gm.eps;
  int lc = S.n_lights;
  int ln = 0;
  if (lc > 0) {
    // sampleOneLight (Scene.hs:109-118) -> estimateDirect (Scene.hs:84-99)
    if (lc > 1) ln = min((int)floorf(lNumU * (float)lc), lc - 1);
    const DLight& l = S.lights[ln];
    // sampleLightMis (Scene.hs:61-69), visibility deferred
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
        storeBands(st.ls, s, lsv);
        Ray sr = smpl.ray;
        storeRay(st.sray, s, sr);
        flags |= VF_SHADOW;
      }
    }
    // sampleBsdfMis (Scene.hs:71-82), the hit deferred as an occlusion
    // query (occlusionSlot above).  An area light's term counts only when
    // the closest hit is its shape, so a ray that misses the shape needs no
    // query unless the term could be NaN; an infinite light's term needs to
    // know whether the ray hits anything.  A point or directional light
    // emits along no ray (le is zero), so its term is f * 0 scaled by the
    // weight: zero whatever the ray meets unless f or the weight is not
    // finite or the ray is degenerate (a NaN sample); only then is the ray
    // traced.
    BsdfSample bm = sampleBsdf(bsdf, wo, lBsdfCompU, lb1, lb2);
    if (!(bm.pdf == 0 || isBlack(bm.f))) {
      float w = powerHeuristic(bm.pdf, lightPdf(A, l, p, bm.wi));
      Ray mr{p, bm.wi, eps, INFINITY};
      float4 rec = hitRecord(false, 0.0f, -1, 0.0f, 0.0f);
      bool query = false;
      if (l.kind == DLIGHT_AREA) {
        const DShape& sh = A.shapes[l.shape];
        float tl, el;
        if (shapeIntersect<false>(sh, transRay(sh.w2o, mr), tl, el, nullptr)) {
          mr.tmax = tl;
          rec = hitRecord(true, tl, S.shape_prim[l.shape], 0.0f, 0.0f);
          query = true;
        }
      }
      if (!query)
        query = l.kind == DLIGHT_INFINITE || !(isfinite(w) && allFinite(bm.f)) ||
                degenerateRay(mr);
      if (query) {
        storeBands(st.bsf, s, bm.f);
        st.bsw[s] = w;
        storeRay(st.mray, s, mr);
        st.mhit[s] = rec;
        flags |= VF_MIS;
        out.mis = true;
      }
    }
  }
  // Russian roulette and the continuation (Path.hs:68-87)
  float pc = depth <= P.rr_depth ? 1.0f : hmin(0.75f, sY(loadBands(st.T, s)));
  float x = rnd1(smp, 3 + 4 * depth);
  if (!(x > pc)) {
    float uc = rnd1(smp, 0 + 4 * depth);
    float ud1, ud2;
    rnd2(smp, 0 + 3 * depth, ud1, ud2);
    BsdfSample bc = sampleBsdf(bsdf, wo, uc, ud1, ud2);
    if (!(bc.pdf == 0 || isBlack(bc.f))) {
      storeBands(st.fc, s, bc.f);
      st.invpc[s] = 1.0f / pc;
      bool spec2 = (bc.type & T_SPEC) != 0;
      storeRay(st.ray, s, Ray{p, bc.wi, spec2 ? -eps : eps, INFINITY});
      flags |= VF_CONT;
    }
  }
  st.vflags[s] = flags | (ln << 8);
  out.shadow = (flags & VF_SHADOW) != 0;
  out.resolve = true;
  return out;
}

// Second half of the vertex (Path.hs:60-87): adds the vertex's radiance once
// its shadow and MIS rays are traced and computes the new throughput.
// Returns true when the path continues, with its throughput and radiance in
// Tn and Ln (the caller stores them); a path that ends is handed to finish(L).
// KEEP_L (paths that stay in their slot): a continuing path that gains no
// radiance here, with a finite throughput, keeps L + T * 0 = L in place: *l_same
// is set and neither L nor Ln is touched.
template <bool KEEP_L = false, class Finish>
__device__ __forceinline__ bool resolveVertex(const DevAccel& A, const DevShading& S,
                                              const Slots& st, int s,
                                              unsigned long long* counters, Finish finish,
                                              Spec& Tn, Spec& Ln, bool* l_same = nullptr) {
  size_t c = st.cap;
  int vf = st.vflags[s];
  int lc = S.n_lights;
  Spec lsv = sConst(0), bsv = sConst(0);
  if ((vf & VF_SHADOW) && st.svis[s]) lsv = loadBands(st.ls, s);
  if (vf & VF_MIS) {
    const DLight& l = S.lights[vf >> 8];
    Ray mr = loadRay7(st.mray, s);
    const float4 mh = st.mhit[s];
    int mp = __float_as_int(mh.y);
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
          HitGeom gm =
              hitGeometry(A, S, mr, mp, mh.x, mh.z, mh.w);
          lr = intLe(S, gm, -mr.d);
          use = true;
        }
      }
    } else {
      lr = lightLe(l, mr.d);
      use = true;
    }
    if (use) bsv = sScale(loadBands(st.bsf, s) * lr, st.bsw[s]);
  }
  Spec ed = lsv + bsv;  // estimateDirect = ls + bs (Scene.hs:95)
  Spec direct = lc == 1 ? ed : (lc > 1 ? sScale(ed, (float)lc) : sConst(0));
  // intl is zero without VF_LE, and 0 + direct is direct (up to the sign of
  // a zero, which the film's sums do not keep)
  Spec lHere = (vf & VF_LE) ? loadBands(st.intl, s) + direct : direct;
  Spec T = loadBands(st.T, s);
  if (KEEP_L && (vf & VF_CONT) && isBlack(lHere) && allFinite(T)) {
    Tn = sScale(loadBands(st.fc, s) * T, st.invpc[s]);
    *l_same = true;
    return true;
  }
  Spec Lr = loadBands(st.L, s) + T * lHere;
  if (vf & VF_CONT) {
    Tn = sScale(loadBands(st.fc, s) * T, st.invpc[s]);
    Ln = Lr;
    return true;
  }
  finish(Lr);
  return false;
}

}  // namespace bgpu
