// Wavefront path integrator on the GPU.
//
// One pass of the reference's sampler renderer (prender/tile,
// Rendering.hs:111-150) with the path integrator (Integrator/Path.hs:30-87):
// every pixel of the filter-padded sample extent gets strata_x*strata_y
// camera paths.  Paths live in SoA slots (throughput and radiance as 16-band
// spectra, band-major), and each bounce is three launches over a queue of
// live slots:
//
//   k_trace   closest hit of the bounce rays (Scene.scIntersect)
//   k_shade   nextVertex (Path.hs:49-87): emission on specular paths, one
//             light sample with its shadow any-hit and its BSDF-sampled MIS
//             closest-hit traversed inline (sampleOneLight/estimateDirect,
//             Scene.hs:184-241), Russian roulette, the continuation sample;
//             live slots are appended to the next queue with one atomic per
//             warp (__ballot_sync/__popc); finished paths are splatted into
//             the film (addSample, Image.hs:250-299) with atomics.
//
// All arithmetic follows the reference's operation order (the file is built
// with -fmad=false); random numbers come from the counter-based generator
// shared with the CPU oracle (see the sampler section below).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dmath.cuh"
#include "dshape.cuh"
#include "integrator.h"
#include "spectrum_tables.h"
#include "trace.cuh"

namespace bgpu {

// ------------------------------------------------------------------ spectra
struct Spec {
  float v[16];
};
__device__ __forceinline__ Spec sConst(float c) {
  Spec s;
#pragma unroll
  for (int i = 0; i < 16; i++) s.v[i] = c;
  return s;
}
__device__ __forceinline__ Spec sLoad(const float* p) {
  Spec s;
#pragma unroll
  for (int i = 0; i < 16; i++) s.v[i] = __ldg(p + i);
  return s;
}
__device__ __forceinline__ Spec operator+(const Spec& a, const Spec& b) {
  Spec s;
#pragma unroll
  for (int i = 0; i < 16; i++) s.v[i] = a.v[i] + b.v[i];
  return s;
}
__device__ __forceinline__ Spec operator-(const Spec& a, const Spec& b) {
  Spec s;
#pragma unroll
  for (int i = 0; i < 16; i++) s.v[i] = a.v[i] - b.v[i];
  return s;
}
__device__ __forceinline__ Spec operator*(const Spec& a, const Spec& b) {
  Spec s;
#pragma unroll
  for (int i = 0; i < 16; i++) s.v[i] = a.v[i] * b.v[i];
  return s;
}
__device__ __forceinline__ Spec sScale(const Spec& a, float f) {
  Spec s;
#pragma unroll
  for (int i = 0; i < 16; i++) s.v[i] = a.v[i] * f;
  return s;
}
__device__ __forceinline__ bool isBlack(const Spec& s) {
  bool b = true;
#pragma unroll
  for (int i = 0; i < 16; i++) b = b && (s.v[i] == 0);
  return b;
}
__device__ __forceinline__ Spec sClamp01(const Spec& a) {
  Spec s;
#pragma unroll
  for (int i = 0; i < 16; i++) s.v[i] = hmax(0.0f, hmin(1.0f, a.v[i]));
  return s;
}

__constant__ float c_cieX[16], c_cieY[16], c_cieZ[16];
__constant__ float c_cieYSum;

// sY (Spectrum.hs:371-373)
__device__ __forceinline__ float sY(const Spec& s) {
  float acc = 0.0f;
#pragma unroll
  for (int i = 0; i < 16; i++) acc = acc + s.v[i] * c_cieY[i];
  return acc / c_cieYSum;
}

// ------------------------------------------------------------------ sampler
// Counter-based generator shared with the CPU oracle: SplitMix64 finaliser
// (Steele, Lea, Flood 2014) keyed by (seed, pass, pixel, sample, dimension);
// stratified dimensions are assigned to pixel samples through Kensler's hash
// permutation (Correlated Multi-Jittered Sampling, 2013), standing in for the
// reference's per-pixel shuffles (Sampling.hs:134-152).
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z ^= z >> 30;
  z *= 0xbf58476d1ce4e5b9ULL;
  z ^= z >> 27;
  z *= 0x94d049bb133111ebULL;
  z ^= z >> 31;
  return z;
}
__device__ __forceinline__ uint64_t pixelKey(uint64_t seed, uint64_t pass, int px, int py) {
  uint64_t k = mix64(seed ^ mix64(pass + 0x9e3779b97f4a7c15ULL));
  return mix64(k ^ (((uint64_t)(uint32_t)px << 32) | (uint64_t)(uint32_t)py));
}
__device__ __forceinline__ uint32_t randU32(uint64_t key, uint32_t n, uint32_t dim) {
  return (uint32_t)(mix64(key ^ mix64(((uint64_t)n << 32) | dim)) >> 32);
}
__device__ __forceinline__ float randF(uint64_t key, uint32_t n, uint32_t dim) {
  return (float)(randU32(key, n, dim) >> 8) * (1.0f / 16777216.0f);
}
__device__ __forceinline__ uint32_t permute(uint32_t i, uint32_t l, uint32_t p) {
  uint32_t w = l - 1;
  w |= w >> 1;
  w |= w >> 2;
  w |= w >> 4;
  w |= w >> 8;
  w |= w >> 16;
  do {
    i ^= p;
    i *= 0xe170893du;
    i ^= p >> 16;
    i ^= (i & w) >> 4;
    i ^= p >> 8;
    i *= 0x0929eb3fu;
    i ^= p >> 23;
    i ^= (i & w) >> 1;
    i *= 1u | p >> 27;
    i *= 0x6935fa69u;
    i ^= (i & w) >> 11;
    i *= 0x74dcb303u;
    i ^= (i & w) >> 2;
    i *= 0x9e501cc3u;
    i ^= (i & w) >> 2;
    i *= 0xc860a3dfu;
    i &= w;
    i ^= i >> 5;
  } while (i >= l);
  return (i + p) % l;
}
enum : uint32_t {
  DIM_PIX_U = 0,
  DIM_PIX_V = 1,
  DIM_LENS_PERM = 2,
  DIM_LENS_U = 3,
  DIM_LENS_V = 4,
  DIM_1D_BASE = 16,
  DIM_2D_BASE = 4096,
  DIM_FRESH_1D = 1u << 20,
  DIM_FRESH_2D = 2u << 20
};
static constexpr float kAlmostOne = 0.9999999403953552f;  // Sampling.hs:154-155

struct Sampler {
  uint64_t key;
  uint32_t n;
  int nu, nv, n1d, n2d;
};
// stratified2D entry i (Sampling.hs:164-171)
__device__ __forceinline__ void strat2D(const Sampler& s, uint32_t i, uint32_t dju, uint32_t djv,
                                        float& u, float& v) {
  float du = 1.0f / (float)s.nu, dv = 1.0f / (float)s.nv;
  uint32_t qu = i / (uint32_t)s.nu, qv = i % (uint32_t)s.nu;
  float ju = randF(s.key, i, dju), jv = randF(s.key, i, djv);
  u = hmin(kAlmostOne, ((float)qu + ju) * du);
  v = hmin(kAlmostOne, ((float)qv + jv) * dv);
}
// rnd' n (Sampling.hs:203-211)
__device__ __forceinline__ float rnd1(const Sampler& s, int n) {
  if (n < s.n1d) {
    uint32_t N = (uint32_t)(s.nu * s.nv);
    uint32_t p = randU32(s.key, 0xffffffffu, DIM_1D_BASE + 2 * n);
    uint32_t st = permute(s.n, N, p);
    float du = 1.0f / (float)N;
    float j = randF(s.key, st, DIM_1D_BASE + 2 * n + 1);
    return hmin(kAlmostOne, ((float)st + j) * du);
  }
  return randF(s.key, s.n, DIM_FRESH_1D | (uint32_t)n);
}
// rnd2D' n (Sampling.hs:213-221)
__device__ __forceinline__ void rnd2(const Sampler& s, int n, float& u, float& v) {
  if (n < s.n2d) {
    uint32_t N = (uint32_t)(s.nu * s.nv);
    uint32_t p = randU32(s.key, 0xffffffffu, DIM_2D_BASE + 4 * n);
    uint32_t st = permute(s.n, N, p);
    strat2D(s, st, DIM_2D_BASE + 4 * n + 1, DIM_2D_BASE + 4 * n + 2, u, v);
    return;
  }
  u = randF(s.key, s.n, DIM_FRESH_2D | (uint32_t)(2 * n));
  v = randF(s.key, s.n, DIM_FRESH_2D | (uint32_t)(2 * n + 1));
}

// ------------------------------------------------------------------ pass constants
struct PassParams {
  uint64_t seed, pass;
  int x0, y0, nx, ny;  // sample extent origin and size (imageWindow', Image.hs:170-176)
  int x1, y1;
  int spp, nu, nv, n1d, n2d;
  int max_depth, rr_depth;
  int width, height;
  float fw, fh;
  uint64_t chunk_base;
};

// ------------------------------------------------------------------ Monte Carlo
// concentricSampleDisk (Montecarlo.hs:389-406)
__device__ __forceinline__ void concentricSampleDisk(float u1, float u2, float& ox, float& oy) {
  float sx = u1 * 2.0f - 1.0f, sy = u2 * 2.0f - 1.0f;
  if (sx == 0 && sy == 0) {
    ox = 0;
    oy = 0;
    return;
  }
  float r, thp;
  if (sx >= -sy) {
    if (sx > sy) {
      r = sx;
      thp = sy > 0 ? sy / sx : 8.0f + sy / sx;
    } else {
      r = sy;
      thp = 2.0f - sx / sy;
    }
  } else if (sx <= sy) {
    r = -sx;
    thp = 4.0f - sy / (-sx);
  } else {
    r = -sy;
    thp = 6.0f + sx / (-sy);
  }
  float theta = thp * kPi / 4.0f;
  ox = r * cosf(theta);
  oy = r * sinf(theta);
}
__device__ __forceinline__ V3 cosineSampleHemisphere(float u1, float u2) {
  float x, y;
  concentricSampleDisk(u1, u2, x, y);
  return V3{x, y, sqrtf(hmax(0.0f, 1.0f - x * x - y * y))};
}
__device__ __forceinline__ V3 uniformSampleSphere(float u1, float u2) {
  float u = u1 * 2.0f - 1.0f;
  float s = sqrtf(1.0f - (u * u));
  float omega = u2 * 2.0f * kPi;
  return V3{s * cosf(omega), s * sinf(omega), u};
}
__device__ __forceinline__ float uniformConePdf(float cosThetaMax) {
  if (cosThetaMax >= 1) return 0;
  return 1.0f / ((2.0f * kPi) * (1.0f - cosThetaMax));
}
__device__ __forceinline__ V3 uniformSampleCone(const LC& c, float cosThetaMax, float u1, float u2) {
  float cosTheta = hlerp(u1, cosThetaMax, 1.0f);
  float sinTheta = sqrtf(1.0f - cosTheta * cosTheta);
  float phi = u2 * (2.0f * kPi);
  float a = cosf(phi) * sinTheta, b = sinf(phi) * sinTheta;
  return V3{c.s.x * a, c.s.y * a, c.s.z * a} + V3{c.t.x * b, c.t.y * b, c.t.z * b} +
         V3{c.n.x * cosTheta, c.n.y * cosTheta, c.n.z * cosTheta};
}
__device__ __forceinline__ float powerHeuristic(float fPdf, float gPdf) {
  float f = 1.0f * fPdf, g = 1.0f * gPdf;
  return (f * f) / (f * f + g * g);
}

// ------------------------------------------------------------------ BSDF
static constexpr float kInvPi = 1.0f / kPi;
static constexpr float kInvTwoPi = 1.0f / (2.0f * kPi);

__device__ __forceinline__ float cosTheta(V3 v) { return v.z; }
__device__ __forceinline__ float absCosTheta(V3 v) { return fabsf(v.z); }
__device__ __forceinline__ float sinTheta2(V3 v) { return hmax(0.0f, 1.0f - v.z * v.z); }
__device__ __forceinline__ float sinTheta(V3 v) { return sqrtf(sinTheta2(v)); }
__device__ __forceinline__ float cosPhi(V3 v) {
  float st = sinTheta(v);
  return st == 0 ? 1.0f : hclamp(v.x / st, -1, 1);
}
__device__ __forceinline__ float sinPhi(V3 v) {
  float st = sinTheta(v);
  return st == 0 ? 0.0f : hclamp(v.y / st, -1, 1);
}
__device__ __forceinline__ bool sameHemisphere(V3 a, V3 b) { return a.z * b.z > 0; }
__device__ __forceinline__ V3 toSameHemisphere(V3 wo, V3 wi) {
  return wo.z < 0 ? V3{wi.x, wi.y, -wi.z} : wi;
}

enum { BX_LAMBERT, BX_OREN, BX_SPEC_REFL, BX_SPEC_TRANS, BX_MICRO };
enum { T_REFL = 1, T_TRANS = 2, T_DIFF = 4, T_GLOSSY = 8, T_SPEC = 16 };
enum { FR_NOOP, FR_DIEL, FR_COND };

struct BxDF {
  int kind, type;
  const float* r;  // spectrum in global memory, null = white
  float A, B;      // Oren-Nayar
  float ei, et;    // dielectric Fresnel / transmission
  float e;         // Blinn exponent
  int fr;
  const float* eta;
  const float* k;
  bool clampR;     // glass: sClamp' of the colour
};
__device__ __forceinline__ Spec bxR(const BxDF& b) {
  if (!b.r) return sConst(1.0f);
  Spec s = sLoad(b.r);
  return b.clampR ? sClamp01(s) : s;
}

// frDielectric (Fresnel.hs:146-180), one value for all bands
__device__ __forceinline__ float frDielScalar(float etai, float etat, float cosi) {
  float c = hmax(0.0f, 1.0f - cosi * cosi);
  float costp = cosi > 0 ? c / (etat * etat) : c * (etat * etat);
  float cost = sqrtf(1.0f - hclamp(costp, 0, 1));
  float ac = fabsf(cosi);
  float eta = etat / etai;
  float rParlp = eta * ac;
  float rParl = (cost - rParlp) / (cost + rParlp);
  float rPerpp = eta * cost;
  float rPerp = (ac - rPerpp) / (ac + rPerpp);
  return (rParl * rParl + rPerp * rPerp) * 0.5f;
}
// r * fr(cosi) (fresnel of the BxDF applied to its colour)
__device__ __forceinline__ Spec rTimesFresnel(const BxDF& b, float cosi) {
  Spec r = bxR(b);
  if (b.fr == FR_NOOP) return r;
  if (b.fr == FR_DIEL) {
    float f = frDielScalar(b.ei, b.et, cosi);
    return r * sConst(f);
  }
  // frConductor (Fresnel.hs:183-195)
  float acosi = fabsf(cosi);
  Spec out;
#pragma unroll
  for (int i = 0; i < 16; i++) {
    float eta = __ldg(b.eta + i), k = __ldg(b.k + i);
    float tmpF = eta * eta + k * k;
    float tmp = (eta * eta + k * k) * (acosi * acosi);
    float ec2 = eta * (2.0f * acosi);
    float a2 = acosi * acosi;
    float rPer2 = (tmpF - ec2 + a2) / (tmpF + ec2 + a2);
    float rPar2 = (tmp - ec2 + 1.0f) / (tmp + ec2 + 1.0f);
    out.v[i] = r.v[i] * ((rPer2 + rPar2) / 2.0f);
  }
  return out;
}

// Blinn (Microfacet.hs:113-195)
__device__ __forceinline__ float mfG(V3 wo, V3 wi, V3 wh) {
  float nDotWh = absCosTheta(wh), nDotWo = absCosTheta(wo), nDotWi = absCosTheta(wi);
  float woDotWh = absDot(wo, wh);
  return hmin(1.0f, hmin(2.0f * nDotWh * nDotWo / woDotWh, 2.0f * nDotWh * nDotWi / woDotWh));
}
__device__ __forceinline__ float blinnPdf(float e, V3 wh) {
  return (e + 1.0f) * powf(absCosTheta(wh), e) * kInvTwoPi;
}
__device__ __forceinline__ float blinnD(float e, V3 wh) {
  return (e + 2.0f) * kInvTwoPi * powf(absCosTheta(wh), e);
}
__device__ __forceinline__ float fixExponent(float e) { return (e > 10000 || isnan(e)) ? 10000.0f : e; }

__device__ __forceinline__ float orenNayarScale(const BxDF& b, V3 wo, V3 wi) {
  float sinti = sinTheta(wi), sinto = sinTheta(wo);
  float sina, tanb;
  if (absCosTheta(wi) > absCosTheta(wo)) {
    sina = sinto;
    tanb = sinti / absCosTheta(wi);
  } else {
    sina = sinti;
    tanb = sinto / absCosTheta(wo);
  }
  float maxcos = 0;
  if (sinti > 1e-4f && sinto > 1e-4f) {
    float sinpi = sinPhi(wi), cospi = cosPhi(wi), sinpo = sinPhi(wo), cospo = cosPhi(wo);
    maxcos = hmax(0.0f, cospi * cospo + sinpi * sinpo);
  }
  return b.A + b.B * maxcos * sina * tanb;
}

// bxdfEval b wo wi
__device__ Spec bxEval(const BxDF& b, V3 wo, V3 wi) {
  switch (b.kind) {
    case BX_LAMBERT: return sScale(bxR(b), kInvPi * absCosTheta(wo));
    case BX_OREN: return sScale(sScale(bxR(b), orenNayarScale(b, wo, wi)), kInvPi * absCosTheta(wo));
    case BX_MICRO: {
      float costo = absCosTheta(wo), costi = absCosTheta(wi);
      if (costi == 0 || costo == 0) return sConst(0);
      V3 whp = wi + wo;
      if (whp.x == 0 && whp.y == 0 && whp.z == 0) return sConst(0);
      V3 wh = normalize(whp);
      if (cosTheta(wh) < 0) return sConst(0);
      float costh = dot(wi, wh);
      float x = blinnD(b.e, wh) * mfG(wo, wi, wh) / (4.0f * costi);
      return sScale(rTimesFresnel(b, costh), x);
    }
    default: return sConst(0);
  }
}
__device__ float bxPdf(const BxDF& b, V3 wo, V3 wi) {
  switch (b.kind) {
    case BX_LAMBERT:
    case BX_OREN: return sameHemisphere(wo, wi) ? kInvPi * absCosTheta(wi) : 0.0f;
    case BX_MICRO: {
      V3 whp = wo + wi;
      if (sqLen(whp) == 0) return 0;
      V3 wh = normalize(whp);
      if (cosTheta(wh) < 0) return 0;
      return blinnPdf(b.e, wh) / (4.0f * absDot(wo, wh));
    }
    default: return 0;
  }
}
__device__ void bxSample(const BxDF& b, V3 wo, float u1, float u2, Spec& f, V3& wi, float& pdf) {
  switch (b.kind) {
    case BX_LAMBERT:
    case BX_OREN: {
      wi = toSameHemisphere(wo, cosineSampleHemisphere(u1, u2));
      if (sameHemisphere(wo, wi)) {
        f = b.kind == BX_LAMBERT ? bxR(b) : sScale(bxR(b), orenNayarScale(b, wo, wi));
        pdf = bxPdf(b, wo, wi);
      } else {
        f = sConst(0);
        pdf = 0;
      }
      return;
    }
    case BX_SPEC_REFL:
      f = rTimesFresnel(b, cosTheta(wo));
      wi = V3{-wo.x, -wo.y, wo.z};
      pdf = 1;
      return;
    case BX_SPEC_TRANS: {
      bool entering = cosTheta(wo) > 0;
      float ei = entering ? b.ei : b.et, et = entering ? b.et : b.ei;
      float sini2 = sinTheta2(wo);
      float eta = ei / et;
      float eta2 = eta * eta;
      float sint2 = eta2 * sini2;
      if (sint2 >= 1) {
        f = sConst(0);
        wi = wo;
        pdf = 0;
        return;
      }
      float c = sqrtf(hmax(0.0f, 1.0f - sint2));
      float cost = entering ? -c : c;
      wi = V3{eta * (-wo.x), eta * (-wo.y), cost};
      float fr = frDielScalar(ei, et, cost);
      Spec t = bxR(b);
#pragma unroll
      for (int i = 0; i < 16; i++) f.v[i] = ((1.0f - fr) * t.v[i]) * eta2;
      pdf = 1;
      return;
    }
    default: {
      float cost = powf(u1, 1.0f / (b.e + 1.0f));
      float sint = sqrtf(hmax(0.0f, 1.0f - cost * cost));
      float phi = u2 * 2.0f * kPi;
      V3 whp{sint * cosf(phi), sint * sinf(phi), cost};
      float ff = powf(cost, b.e) * kInvTwoPi;
      float d = (b.e + 2.0f) * ff;
      float p = (b.e + 1.0f) * ff;
      V3 wh = cosTheta(whp) < 0 ? -whp : whp;
      wi = sv(2.0f * dot(wo, wh), wh) - wo;
      float costH = dot(wo, wh);
      float fact = d * fabsf(costH) / p * mfG(wo, wi, wh);
      if (sameHemisphere(wo, wi)) {
        f = sScale(rTimesFresnel(b, costH), fact / absCosTheta(wi));
        pdf = p / (4.0f * fabsf(costH));
      } else {
        f = sConst(0);
        wi = wo;
        pdf = 0;
      }
      return;
    }
  }
}

struct Bsdf {
  BxDF c[2];
  int n;
  LC cs;
  V3 p, ng;
};

// mkBsdf' with the material's BxDFs (Material.hs:228-292)
__device__ Bsdf materialBsdf(const DMaterial* __restrict__ mats, int mi, V3 dgg_n, V3 dgs_p,
                             V3 dgs_n, V3 dgs_dpdu) {
  const DMaterial& m = mats[mi];
  Bsdf b;
  b.n = 0;
  V3 sn = normalize(dgs_dpdu);
  b.cs = LC{sn, cross(dgs_n, sn), dgs_n};
  b.p = dgs_p;
  b.ng = dgg_n;
  BxDF x;
  x.r = nullptr;
  x.A = x.B = x.ei = x.et = x.e = 0;
  x.fr = FR_NOOP;
  x.eta = x.k = nullptr;
  x.clampR = false;
  int kind = m.kind;
  float sigma = m.sigma, rough = m.rough, ior = m.ior;
  if (kind == BLING_MAT_MATTE) {
    x.type = T_REFL | T_DIFF;
    x.r = m.kd;
    if (sigma == 0) {
      x.kind = BX_LAMBERT;
    } else {
      x.kind = BX_OREN;
      float s = hclamp(sigma, 0, 1);
      float sig2 = s * s;
      x.A = 1.0f - (sig2 / (2.0f * (sig2 + 0.33f)));
      x.B = 0.45f * sig2 / (sig2 + 0.09f);
    }
    b.c[b.n++] = x;
  } else if (kind == BLING_MAT_PLASTIC) {
    x.kind = BX_LAMBERT;
    x.type = T_REFL | T_DIFF;
    x.r = m.kd;
    b.c[b.n++] = x;
    BxDF y = x;
    y.kind = BX_MICRO;
    y.type = T_REFL | T_GLOSSY;
    y.r = m.ks;
    y.e = fixExponent(1.0f / rough);
    y.fr = FR_DIEL;
    y.ei = 1.0f;
    y.et = 1.5f;
    b.c[b.n++] = y;
  } else if (kind == BLING_MAT_METAL) {
    x.kind = BX_MICRO;
    x.type = T_REFL | T_GLOSSY;
    x.r = nullptr;
    x.e = fixExponent(1.0f / rough);
    x.fr = FR_COND;
    x.eta = m.eta;
    x.k = m.k;
    b.c[b.n++] = x;
  } else {
    x.kind = BX_SPEC_REFL;
    x.type = T_REFL | T_SPEC;
    x.r = m.ks;
    x.clampR = true;
    x.fr = FR_DIEL;
    x.ei = 1.0f;
    x.et = ior;
    b.c[b.n++] = x;
    BxDF y = x;
    y.kind = BX_SPEC_TRANS;
    y.type = T_TRANS | T_SPEC;
    y.r = m.kt;
    y.clampR = true;
    y.fr = FR_NOOP;
    y.ei = 1.0f;
    y.et = ior;
    b.c[b.n++] = y;
  }
  return b;
}

struct BsdfSample {
  int type;
  float pdf;
  Spec f;
  V3 wi;
};

// sampleBsdf'' False bxdfAll (Reflection.hs:278-316)
__device__ BsdfSample sampleBsdf(const Bsdf& b, V3 woW, float uComp, float u1, float u2) {
  BsdfSample out;
  out.type = T_REFL | T_DIFF;
  out.pdf = 0;
  out.f = sConst(0);
  out.wi = V3{0, 1, 0};
  if (b.n == 0) return out;
  V3 wo = worldToLocal(b.cs, woW);
  int cntm = b.n;
  float cntf = (float)cntm;
  float invCnt = 1.0f / cntf;
  int sNum = max(0, min(cntm - 1, (int)floorf(uComp * cntf)));
  const BxDF& bx = b.c[sNum];
  Spec fSample;
  V3 wi;
  float pdfp;
  bxSample(bx, wo, u1, u2, fSample, wi, pdfp);
  V3 wiW = localToWorld(b.cs, wi);
  float sideTest = dot(wiW, b.ng) / dot(woW, b.ng);
  if (pdfp == 0 || sideTest == 0) return out;
  bool wantTrans = sideTest < 0;
  bool ok = wantTrans ? (bx.type & T_TRANS) != 0 : (bx.type & T_REFL) != 0;
  if (!ok) return out;
  out.type = bx.type;
  out.wi = wiW;
  if (bx.type & T_SPEC) {
    out.pdf = pdfp * invCnt;
    out.f = sScale(fSample, cntf);
    return out;
  }
  if (cntm == 1) {
    out.pdf = pdfp;
    out.f = fSample;
    return out;
  }
  float others = 0.0f;
  for (int i = 0; i < cntm; i++)
    if (i != sNum) others = others + bxPdf(b.c[i], wo, wi);
  float pdf = (pdfp + others) * invCnt;
  Spec fOthers = sConst(0);
  for (int i = 0; i < cntm; i++) {
    if (i == sNum) continue;
    bool ok2 = wantTrans ? (b.c[i].type & T_TRANS) != 0 : (b.c[i].type & T_REFL) != 0;
    if (ok2) fOthers = fOthers + bxEval(b.c[i], wi, wo);
  }
  out.pdf = pdf;
  out.f = sScale(sScale(fSample, pdfp) + fOthers, 1.0f / pdf);
  return out;
}
// evalBsdf False (Reflection.hs:318-332)
__device__ Spec evalBsdf(const Bsdf& b, V3 woW, V3 wiW) {
  float cosWo = dot(woW, b.ng);
  float sideTest = dot(wiW, b.ng) / cosWo;
  if (sideTest == 0) return sConst(0);
  if (fabsf(cosWo) < 1e-5f) return sConst(0);
  bool wantTrans = sideTest < 0;
  V3 wo = worldToLocal(b.cs, woW), wi = worldToLocal(b.cs, wiW);
  Spec f = sConst(0);
  for (int i = 0; i < b.n; i++) {
    bool ok = wantTrans ? (b.c[i].type & T_TRANS) != 0 : (b.c[i].type & T_REFL) != 0;
    if (ok) f = f + bxEval(b.c[i], wi, wo);
  }
  return f;
}
// bsdfPdf (Reflection.hs:251-257)
__device__ float bsdfPdf(const Bsdf& b, V3 woW, V3 wiW) {
  if (b.n == 0) return 0;
  V3 wo = worldToLocal(b.cs, woW), wi = worldToLocal(b.cs, wiW);
  float s = 0.0f;
  for (int i = 0; i < b.n; i++) s = s + bxPdf(b.c[i], wo, wi);
  return s / (float)b.n;
}

// ------------------------------------------------------------------ geometry at hits
struct HitGeom {
  V3 p, n;           // intGeometry (world)
  V3 sp, sn, sdpdu;  // shading geometry
  float eps;
  int material;
  int light_id;      // area light of the primitive, -1 if none
  int shape;         // shape index or -1
};

// builds the intersection's DG for primitive `prim` hit at t (TriangleMesh.hs:182-207,
// Geometry.hs:33-36, triangleShadingGeometry TriangleMesh.hs:122-134)
__device__ HitGeom hitGeometry(const DevAccel& A, const DevShading& S, const Ray& r, int prim,
                               float t, float b1, float b2) {
  HitGeom g;
  int2 info = __ldg(S.prim_info + prim);
  if (info.x < 0) {
    const DShape& sh = A.shapes[~info.x];
    Ray ro = transRay(sh.w2o, r);
    float tt, e;
    DGeo dg;
    ro.tmax = INFINITY;
    shapeIntersect<true>(sh, ro, tt, e, &dg);
    g.eps = e;
    g.p = transPoint(sh.o2w, dg.p);
    g.n = normalize(transNormal(sh.w2o, dg.n));
    g.sdpdu = transVector(sh.o2w, dg.dpdu);
    g.sp = g.p;
    g.sn = g.n;
    g.material = sh.material;
    g.light_id = sh.light_id;
    g.shape = ~info.x;
    return g;
  }
  const DMesh& m = S.meshes[info.x];
  int t3 = 3 * info.y;
  int o1 = __ldg(m.idx + t3), o2 = __ldg(m.idx + t3 + 1), o3 = __ldg(m.idx + t3 + 2);
  V3 p1{__ldg(m.verts + 3 * o1), __ldg(m.verts + 3 * o1 + 1), __ldg(m.verts + 3 * o1 + 2)};
  V3 p2{__ldg(m.verts + 3 * o2), __ldg(m.verts + 3 * o2 + 1), __ldg(m.verts + 3 * o2 + 2)};
  V3 p3{__ldg(m.verts + 3 * o3), __ldg(m.verts + 3 * o3 + 1), __ldg(m.verts + 3 * o3 + 2)};
  float uv00 = 0, uv01 = 0, uv10 = 1, uv11 = 0, uv20 = 1, uv21 = 1;
  if (m.uvs) {
    uv00 = __ldg(m.uvs + 2 * o1);
    uv01 = __ldg(m.uvs + 2 * o1 + 1);
    uv10 = __ldg(m.uvs + 2 * o2);
    uv11 = __ldg(m.uvs + 2 * o2 + 1);
    uv20 = __ldg(m.uvs + 2 * o3);
    uv21 = __ldg(m.uvs + 2 * o3 + 1);
  }
  V3 e1 = p2 - p1, e2 = p3 - p1;
  float du1 = uv00 - uv20, du2 = uv10 - uv20, dv1 = uv01 - uv21, dv2 = uv11 - uv21;
  V3 dp1 = p1 - p3, dp2 = p2 - p3;
  float determinant = du1 * dv2 - dv1 * du2;
  V3 dpdu, dpdv;
  if (determinant == 0) {
    LC c = coordinateSystem(normalize(cross(e1, e2)));
    dpdu = c.s;
    dpdv = c.t;
  } else {
    float invDet = 1.0f / determinant;
    dpdu = sv(invDet, sv(dv2, dp1) - sv(dv1, dp2));
    dpdv = sv(invDet, sv(-du2, dp1) + sv(du1, dp2));
  }
  g.p = rayAt(r, t);
  g.n = normalize(cross(dpdu, dpdv));
  g.eps = 1e-3f * t;
  g.sp = g.p;
  g.sn = g.n;
  g.sdpdu = dpdu;
  g.material = m.material;
  g.light_id = -1;
  g.shape = -1;
  if (m.normals) {
    V3 n0{__ldg(m.normals + 3 * o1), __ldg(m.normals + 3 * o1 + 1), __ldg(m.normals + 3 * o1 + 2)};
    V3 n1{__ldg(m.normals + 3 * o2), __ldg(m.normals + 3 * o2 + 1), __ldg(m.normals + 3 * o2 + 2)};
    V3 n2{__ldg(m.normals + 3 * o3), __ldg(m.normals + 3 * o3 + 1), __ldg(m.normals + 3 * o3 + 2)};
    float b0 = 1.0f - b1 - b2;
    V3 nsp = sv(b0, n0) + sv(b1, n1) + sv(b2, n2);
    const float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    V3 ns = normalize(transNormal(ident, nsp));
    V3 ssp = normalize(dpdu);
    V3 tsp = cross(ssp, ns);
    V3 ss;
    if (sqLen(tsp) > 0) {
      ss = cross(normalize(tsp), ns);
    } else {
      ss = coordinateSystem(ns).s;
    }
    g.sn = ns;
    g.sdpdu = ss;
  }
  return g;
}

// ------------------------------------------------------------------ lights
__device__ __forceinline__ bool insideSphere(float r, V3 p) { return sqLen(p) - r * r < 1e-4f; }

__device__ void sampleShapeP(const DShape& s, float u1, float u2, V3& p, V3& n) {
  switch (s.kind) {
    case SHAPE_BOX: {
      int axis = min(2, (int)floorf(u1 * 3.0f));
      float u1p = (u1 - (float)axis / 3.0f) * 3.0f;
      int nf = min(1, (int)floorf(u2 * 2.0f));
      float u2p = (u2 - (float)nf / 2.0f) * 2.0f;
      n = setComp(axis, (float)nf * 2.0f - 1.0f, v3(0, 0, 0));
      int oa0 = (axis + 1) % 3, oa1 = (axis + 2) % 3;
      V3 pmin{s.p[0], s.p[1], s.p[2]}, pmax{s.p[3], s.p[4], s.p[5]};
      V3 base = nf == 0 ? pmin : pmax;
      p = setComp(oa0, hlerp(u1p, comp(pmin, oa0), comp(pmax, oa0)),
                  setComp(oa1, hlerp(u2p, comp(pmin, oa1), comp(pmax, oa1)), base));
      return;
    }
    case SHAPE_CYLINDER: {
      float z = hlerp(u1, s.p[1], s.p[2]);
      float phi = hlerp(u2, 0, 2.0f * kPi);
      p = V3{s.p[0] * cosf(phi), s.p[0] * sinf(phi), z};
      n = normalize(V3{p.x, p.y, 0});
      return;
    }
    case SHAPE_DISK: {
      float r = hlerp(u1, s.p[2], s.p[1]);
      float phi = hlerp(u2, 0, s.p[3]);
      p = V3{r * cosf(phi), r * sinf(phi), s.p[0]};
      n = V3{0, 0, -1};
      return;
    }
    case SHAPE_QUAD:
      p = V3{hlerp(u1, -s.p[0], s.p[0]), hlerp(u2, -s.p[1], s.p[1]), 0};
      n = V3{0, 0, -1};
      return;
    default: {
      V3 q = uniformSampleSphere(u1, u2);
      p = q * V3{s.p[0], s.p[0], s.p[0]};
      n = q;
      return;
    }
  }
}
__device__ void sampleShape(const DShape& s, V3 pt, float u1, float u2, V3& ps, V3& ns) {
  if (s.kind == SHAPE_SPHERE && !insideSphere(s.p[0], pt)) {
    float r = s.p[0];
    V3 dn = normalize(-pt);
    LC cs = coordinateSystem(dn);
    float cosThetaMax = sqrtf(hmax(0.0f, 1.0f - (r * r) / sqLen(pt)));
    V3 d = uniformSampleCone(cs, cosThetaMax, u1, u2);
    Ray ray{pt, d, 0, INFINITY};
    float t, e;
    ps = shapeIntersect<false>(s, ray, t, e, nullptr) ? rayAt(ray, t) : dn * V3{r, r, r};
    ns = normalize(ps);
    return;
  }
  sampleShapeP(s, u1, u2, ps, ns);
}
__device__ float shapePdf(const DShape& s, V3 p, V3 wi) {
  if (s.kind == SHAPE_SPHERE && !insideSphere(s.p[0], p)) {
    float r = s.p[0];
    float sinThetaMax2 = r * r / sqLen(p);
    float cosThetaMax = sqrtf(hmax(0.0f, 1.0f - sinThetaMax2));
    return uniformConePdf(cosThetaMax);
  }
  Ray r{p, wi, 1e-3f, INFINITY};
  float t, e;
  DGeo dg;
  if (!shapeIntersect<true>(s, r, t, e, &dg)) return 0;
  float pd = sqLen(p - rayAt(r, t)) / (absDot(dg.n, -wi) * shapeArea(s));
  return isinf(pd) ? 0.0f : pd;
}

__device__ __forceinline__ float sphericalTheta(V3 v) { return acosf(hmax(-1.0f, hmin(1.0f, v.z))); }
__device__ __forceinline__ float sphericalPhi(V3 v) {
  float p = hatan2(v.y, v.x);
  return p < 0 ? p + 2.0f * kPi : p;
}
__device__ __forceinline__ const float* envTexel(const DLight& l, float u, float v) {
  int x = (int)floorf(u * (float)l.env_w), y = (int)floorf(v * (float)l.env_h);
  x = max(0, min(l.env_w - 1, x));
  y = max(0, min(l.env_h - 1, y));
  return l.env + 16 * ((size_t)y * l.env_w + x);
}
// upperBound + sampleContinuous1D (Montecarlo.hs:282-301); findIndex (>= u)
// on a non-decreasing CDF is its lower bound
__device__ void sampleContinuous1D(const float* func, const float* cdf, int n, float fi, float u,
                                   float& x, float& pdf, int& off) {
  int lo = 0, hi = n + 1;  // first index with cdf >= u, n + 1 if none
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (__ldg(cdf + mid) >= u)
      hi = mid;
    else
      lo = mid + 1;
  }
  int xx = lo == n + 1 ? n : lo - 1;
  off = min(n - 1, max(0, xx));
  pdf = fi == 0 ? 0 : __ldg(func + off) / fi;
  float c0 = __ldg(cdf + off), c1 = __ldg(cdf + off + 1);
  float du = (u - c0) / (c1 - c0);
  x = ((float)off + du) / (float)n;
}

struct LightSample {
  Spec li;
  V3 wi;
  Ray ray;
  float pdf;
  bool delta;
};

__device__ LightSample lightSample(const DevAccel& A, const DevShading& S, const DLight& l, V3 p,
                                   float eps, V3 n, float u1, float u2) {
  LightSample ls;
  ls.delta = false;
  if (l.kind == DLIGHT_AREA) {
    const DShape& s = A.shapes[l.shape];
    V3 pl = transPoint(s.w2o, p);
    V3 ps, ns;
    sampleShape(s, pl, u1, u2, ps, ns);
    V3 wi = normalize(ps - pl);
    ls.li = dot(ns, wi) < 0 ? sLoad(S.shape_emission + 16 * l.shape) : sConst(0);
    ls.wi = transVector(s.o2w, wi);
    ls.pdf = shapePdf(s, pl, wi);
    Ray rl{pl, wi, eps, sqrtf(sqLen(ps - pl)) - eps};
    ls.ray = transRay(s.o2w, rl);
    return ls;
  }
  V3 lv{l.vec[0], l.vec[1], l.vec[2]};
  if (l.kind == DLIGHT_DIRECTIONAL) {
    ls.li = sScale(sLoad(l.spec), absDot(n, lv));
    ls.wi = lv;
    ls.ray = Ray{p, lv, eps, INFINITY};
    ls.pdf = 1;
    ls.delta = true;
    return ls;
  }
  if (l.kind == DLIGHT_POINT) {
    ls.li = sScale(sLoad(l.spec), 1.0f / sqLen(lv - p));
    ls.wi = normalize(lv - p);
    ls.ray = Ray{p, lv - p, eps, INFINITY};
    ls.pdf = 1;
    ls.delta = true;
    return ls;
  }
  // infinite (Light.hs:130-141), sampleContinuous2D (Montecarlo.hs:319-322)
  float v, pdf1, u, pdf0;
  int im, iu;
  sampleContinuous1D(l.cond_int, l.marg_cdf, l.env_h, l.marg_int, u2, v, pdf1, im);
  sampleContinuous1D(l.cond_func + (size_t)im * l.env_w, l.cond_cdf + (size_t)im * (l.env_w + 1),
                     l.env_w, __ldg(l.cond_int + im), u1, u, pdf0, iu);
  float mapPdf = pdf0 * pdf1;
  ls.li = sConst(0);
  ls.wi = V3{0, 1, 0};
  ls.ray = Ray{V3{0, 0, 0}, V3{0, 1, 0}, 0, 1};
  ls.pdf = 0;
  if (mapPdf == 0) return ls;
  float phi = u * 2.0f * kPi, theta = v * kPi;
  float sint = sinf(theta);
  if (sint == 0) return ls;
  ls.li = sLoad(envTexel(l, u, v));
  V3 dl{sinf(theta) * cosf(phi), sinf(theta) * sinf(phi), cosf(theta)};
  ls.wi = transVector(l.l2w, dl);
  ls.ray = Ray{p, ls.wi, eps, INFINITY};
  ls.pdf = mapPdf / (2.0f * kPi * kPi * sint);
  return ls;
}
// le (Light.hs:98-106)
__device__ Spec lightLe(const DLight& l, V3 d) {
  if (l.kind != DLIGHT_INFINITE) return sConst(0);
  V3 wh = normalize(transVector(l.w2l, d));
  float phi = sphericalPhi(wh), theta = sphericalTheta(wh);
  return sLoad(envTexel(l, phi / (2.0f * kPi), theta / kPi));
}
// pdf (Light.hs:215-229)
__device__ float lightPdf(const DevAccel& A, const DLight& l, V3 p, V3 wi) {
  if (l.kind == DLIGHT_AREA) {
    const DShape& s = A.shapes[l.shape];
    return shapePdf(s, transPoint(s.w2o, p), transVector(s.w2o, wi));
  }
  if (l.kind != DLIGHT_INFINITE) return 0;
  V3 d = transVector(l.w2l, wi);
  float theta = sphericalTheta(d), phi = sphericalPhi(d);
  float sint = sinf(theta);
  if (sint == 0) return 0;
  float u = phi / (2.0f * kPi), v = theta / kPi;
  int nu = l.env_w, nv = l.env_h;
  int iu = max(0, min(nu - 1, (int)floorf(u * (float)nu)));
  int iv = max(0, min(nv - 1, (int)floorf(v * (float)nv)));
  float ci = __ldg(l.cond_int + iv);
  float pd;
  if (l.marg_int * ci == 0)
    pd = 0;
  else
    pd = (__ldg(l.cond_func + (size_t)iv * nu + iu) * ci) / (ci * l.marg_int);
  return pd / (2.0f * kPi * kPi * sint);
}

// ------------------------------------------------------------------ film
__constant__ float c_filter[256];

// addSample (Image.hs:250-299) into the tile image of the sample's tile
// (mkImageTile/addTile, Image.hs:108-120,178-199): the footprint is clipped to
// the tile's pixel range and to the film.
__device__ void filmAdd(float* __restrict__ film, const PassParams& P, int ix, int iy, float sx,
                        float sy, const Spec& L, unsigned long long* nonfinite) {
  bool bad = false;
#pragma unroll
  for (int i = 0; i < 16; i++) bad = bad || isnan(L.v[i]) || isinf(L.v[i]);
  if (bad) {
    atomicAdd(nonfinite, 1ull);
    return;
  }
  float a = 0, b = 0, c = 0;
#pragma unroll
  for (int i = 0; i < 16; i++) {
    a = a + c_cieX[i] * L.v[i];
    b = b + c_cieY[i] * L.v[i];
    c = c + c_cieZ[i] * L.v[i];
  }
  float smx = a / c_cieYSum, smy = b / c_cieYSum, smz = c / c_cieYSum;
  // tile of (ix, iy) (splitWindow, Sampling.hs:55-58)
  int txs = P.x0 + ((ix - P.x0) / 16) * 16, tys = P.y0 + ((iy - P.y0) / 16) * 16;
  int txe = min(txs + 15, P.x1), tye = min(tys + 15, P.y1);
  int ox = max(0, txs), oy = max(0, tys);
  int tw = txe - ox + (int)floorf(0.5f + P.fw), th = tye - oy + (int)floorf(0.5f + P.fh);
  float fw = P.fw, fh = P.fh;
  float ifw = 1.0f / fw, ifh = 1.0f / fw;  // sic (Image.hs:263)
  float dx = sx - 0.5f, dy = sy - 0.5f;
  int x0 = max(ox, (int)ceilf(dx - fw));
  int x1 = min(ox + tw - 1, (int)floorf(dx + fw));
  int y0 = max(oy, (int)ceilf(dy - fh));
  int y1 = min(oy + th - 1, (int)floorf(dy + fh));
  x1 = min(x1, P.width - 1);
  y1 = min(y1, P.height - 1);
  for (int y = y0; y <= y1; y++) {
    float fy = fabsf(((float)y - dy) * ifh * 16.0f);
    int iyf = min((int)floorf(fy), 15);
    for (int x = x0; x <= x1; x++) {
      float fx = fabsf(((float)x - dx) * ifw * 16.0f);
      int ixf = min((int)floorf(fx), 15);
      float w = c_filter[iyf * 16 + ixf];
      float* px = film + 4 * ((size_t)y * P.width + x);
      atomicAdd(px, w);
      atomicAdd(px + 1, smx * w);
      atomicAdd(px + 2, smy * w);
      atomicAdd(px + 3, smz * w);
    }
  }
}

// ------------------------------------------------------------------ kernels
struct Slots {
  float* T;
  float* L;
  float* ray;
  float* hit_t;
  int32_t* hit_prim;
  float* hit_b;
  size_t cap;
};

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
    size_t c = st.cap;
    st.ray[i] = ray.o.x;
    st.ray[c + i] = ray.o.y;
    st.ray[2 * c + i] = ray.o.z;
    st.ray[3 * c + i] = ray.d.x;
    st.ray[4 * c + i] = ray.d.y;
    st.ray[5 * c + i] = ray.d.z;
    st.ray[6 * c + i] = 0.0f;
#pragma unroll
    for (int b = 0; b < 16; b++) {
      st.T[b * c + i] = 1.0f;
      st.L[b * c + i] = 0.0f;
    }
    queue[i] = (int32_t)i;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    counters[0] = (unsigned long long)count;
    counters[1] = 0;
  }
}

__device__ __forceinline__ Ray loadSlotRay(const Slots& st, int s) {
  size_t c = st.cap;
  return Ray{V3{st.ray[s], st.ray[c + s], st.ray[2 * c + s]},
             V3{st.ray[3 * c + s], st.ray[4 * c + s], st.ray[5 * c + s]}, fabsf(st.ray[6 * c + s]),
             INFINITY};
}

// closest hit of the queued bounce rays (scIntersect), persistent warps that
// take queue entries from counters[5] (zeroed before each launch)
__global__ void __launch_bounds__(128) k_trace(DevAccel A, Slots st, const int32_t* __restrict__ queue,
                                               const unsigned long long* __restrict__ qcount,
                                               unsigned long long* __restrict__ counters) {
  int64_t n = (int64_t)*qcount;
  traceWarpPersistent<false>(
      A, n, counters + 5, [&](int64_t q) { return loadSlotRay(st, queue[q]); },
      [&](int64_t q, const RayQueryResult& res) {
        int s = queue[q];
        st.hit_t[s] = res.t;
        st.hit_prim[s] = res.hit ? res.prim : -1;
        st.hit_b[2 * s] = res.b1;
        st.hit_b[2 * s + 1] = res.b2;
      });
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(counters + 2, (unsigned long long)n);
}

static unsigned traceGrid(int sms) {
  static int per_sm = 0;
  if (!per_sm) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace, 128, 0);
    per_sm = std::max(1, per_sm);
  }
  return (unsigned)(std::max(1, sms) * per_sm);
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

// intLe (Primitive.hs:68-76) + lEmit (Light.hs:85-96)
__device__ __forceinline__ Spec intLe(const DevShading& S, const HitGeom& g, V3 wo) {
  if (g.light_id < 0) return sConst(0);
  return dot(g.n, wo) > 0 ? sLoad(S.shape_emission + 16 * g.shape) : sConst(0);
}

// estimateDirect (Scene.hs:207-222) with its two traversals inline
__device__ Spec estimateDirect(const DevAccel& A, const DevShading& S, int li, V3 p, float eps,
                               V3 n, V3 wo, const Bsdf& bsdf, float ld1, float ld2, float ubc,
                               float ub1, float ub2, unsigned& nclosest, unsigned& nany) {
  const DLight& l = S.lights[li];
  Spec ls = sConst(0);
  {
    LightSample smp = lightSample(A, S, l, p, eps, n, ld1, ld2);
    if (!(smp.pdf == 0 || isBlack(smp.li))) {
      Spec f = evalBsdf(bsdf, wo, smp.wi);
      if (!isBlack(f)) {
        float t, b1, b2;
        int prim;
        nany++;
        if (!traverse<true>(A, smp.ray, t, prim, b1, b2)) {
          if (smp.delta)
            ls = sScale(f * smp.li, 1.0f / smp.pdf);
          else {
            float w = powerHeuristic(smp.pdf, bsdfPdf(bsdf, wo, smp.wi));
            ls = sScale(f * smp.li, w / smp.pdf);
          }
        }
      }
    }
  }
  Spec bs = sConst(0);
  {
    BsdfSample b = sampleBsdf(bsdf, wo, ubc, ub1, ub2);
    if (!(b.pdf == 0 || isBlack(b.f))) {
      Ray ray{p, b.wi, eps, INFINITY};
      float t, b1, b2;
      int prim;
      nclosest++;
      bool h = traverse<false>(A, ray, t, prim, b1, b2);
      bool use = false;
      Spec lr;
      if (h) {
        if (l.kind == DLIGHT_AREA) {
          int2 info = __ldg(S.prim_info + prim);
          if (info.x < 0 && ~info.x == l.shape) {  // Eq Light: same area light
            HitGeom g = hitGeometry(A, S, ray, prim, t, b1, b2);
            lr = intLe(S, g, -b.wi);
            use = true;
          }
        }
      } else {
        lr = lightLe(l, ray.d);
        use = true;
      }
      if (use) {
        float lPdf = lightPdf(A, l, p, b.wi);
        bs = sScale(b.f * lr, powerHeuristic(b.pdf, lPdf));
      }
    }
  }
  return ls + bs;
}

// warp-aggregated append of live slots to the next queue
__device__ __forceinline__ void queueAppend(bool live, int slot, int32_t* __restrict__ queue,
                                            unsigned long long* count) {
  const unsigned mask = 0xffffffffu;  // every lane of the warp reaches this point
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

// one vertex of every queued path (nextVertex, Path.hs:41-87)
__global__ void k_shade(DevAccel A, DevShading S, PassParams P, Slots st, int depth,
                        const int32_t* __restrict__ qin, const unsigned long long* __restrict__ qcount,
                        int32_t* __restrict__ qout, unsigned long long* __restrict__ qout_count,
                        float* __restrict__ film, unsigned long long* __restrict__ counters) {
  int64_t n = (int64_t)*qcount;
  unsigned nclosest = 0, nany = 0;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t nround = (n + stride - 1) / stride * stride;  // whole warps stay converged for the append
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nround; q += stride) {
    bool live = false;
    int s = 0;
    if (q < n) {
      s = qin[q];
      // slots never move: slot s of a chunk holds sample chunk_base + s
      uint64_t g = P.chunk_base + (uint64_t)s;
      int ix, iy;
      uint32_t sn;
      decodeSample(P, g, ix, iy, sn);
      Sampler smp = mkSampler(P, ix, iy, sn);
      Ray ray = loadSlotRay(st, s);
      int prim = st.hit_prim[s];
      Spec T = loadBands(st.T, st.cap, s);
      Spec Lr = loadBands(st.L, st.cap, s);
      // the specular flag travels in the sign bit of the stored tmin (tmin >= 0)
      bool specular = depth == 0 || signbit(st.ray[6 * st.cap + s]);
      bool done = false;
      if (prim < 0) {
        if (specular) {
          Spec sum = sConst(0);
          for (int k = 0; k < S.n_lights; k++) sum = sum + lightLe(S.lights[k], ray.d);
          Lr = Lr + T * sum;
        }
        done = true;
      } else if (depth == P.max_depth) {
        done = true;
      } else {
        float thit = st.hit_t[s], b1 = st.hit_b[2 * s], b2 = st.hit_b[2 * s + 1];
        float lNumU = rnd1(smp, 1 + 4 * depth);
        float ld1, ld2;
        rnd2(smp, 1 + 3 * depth, ld1, ld2);
        float lBsdfCompU = rnd1(smp, 2 + 4 * depth);
        float lb1, lb2;
        rnd2(smp, 2 + 3 * depth, lb1, lb2);
        HitGeom g = hitGeometry(A, S, ray, prim, thit, b1, b2);
        V3 rd = ray.d;
        Spec intl = specular ? intLe(S, g, rd) : sConst(0);
        V3 wo = -rd;
        Bsdf bsdf = materialBsdf(S.materials, g.material, g.n, g.sp, g.sn, g.sdpdu);
        V3 nn = bsdf.cs.n, p = bsdf.p;
        float eps = g.eps;
        Spec direct = sConst(0);
        int lc = S.n_lights;
        if (lc == 1) {
          direct = estimateDirect(A, S, 0, p, eps, nn, wo, bsdf, ld1, ld2, lBsdfCompU, lb1, lb2,
                                  nclosest, nany);
        } else if (lc > 1) {
          int ln = min((int)floorf(lNumU * (float)lc), lc - 1);
          direct = sScale(estimateDirect(A, S, ln, p, eps, nn, wo, bsdf, ld1, ld2, lBsdfCompU, lb1,
                                         lb2, nclosest, nany),
                          (float)lc);
        }
        Spec lHere = intl + direct;
        Lr = Lr + T * lHere;
        float pc = depth <= P.rr_depth ? 1.0f : hmin(0.75f, sY(T));
        float x = rnd1(smp, 3 + 4 * depth);
        if (x > pc) {
          done = true;
        } else {
          float uc = rnd1(smp, 0 + 4 * depth);
          float ud1, ud2;
          rnd2(smp, 0 + 3 * depth, ud1, ud2);
          BsdfSample bs = sampleBsdf(bsdf, wo, uc, ud1, ud2);
          if (bs.pdf == 0 || isBlack(bs.f)) {
            done = true;
          } else {
            T = sScale(bs.f * T, 1.0f / pc);
            bool spec2 = (bs.type & T_SPEC) != 0;
            size_t c = st.cap;
            st.ray[s] = p.x;
            st.ray[c + s] = p.y;
            st.ray[2 * c + s] = p.z;
            st.ray[3 * c + s] = bs.wi.x;
            st.ray[4 * c + s] = bs.wi.y;
            st.ray[5 * c + s] = bs.wi.z;
            st.ray[6 * c + s] = spec2 ? -eps : eps;  // eps >= 0; sign = specular
            storeBands(st.T, st.cap, s, T);
            live = true;
          }
        }
      }
      if (done) {
        float sx, sy, lu, lv;
        pixelSample(P, smp, ix, iy, sx, sy, lu, lv);
        filmAdd(film, P, ix, iy, sx, sy, Lr, counters + 4);
      } else {
        storeBands(st.L, st.cap, s, Lr);
      }
    }
    queueAppend(live, s, qout, qout_count);
  }
  if (nclosest) atomicAdd(counters + 2, (unsigned long long)nclosest);
  if (nany) atomicAdd(counters + 3, (unsigned long long)nany);
}

__global__ void k_reset_count(unsigned long long* c) { *c = 0; }

// ------------------------------------------------------------------ host side
namespace {

float fbits(uint32_t b) {
  float f;
  memcpy(&f, &b, 4);
  return f;
}

// evalFilter (Filter.hs:68-96) and mkTableFilter (Image.hs:48-61), host
float evalFilterHost(int kind, const float* fp, float x, float y) {
  switch (kind) {
    case BLING_FILTER_GAUSS: {
      float w = fp[0], h = fp[1], a = fp[2];
      float ex = expf(-a * w * w), ey = expf(-a * h * h);
      float gx = hmax(0.0f, expf(-a * x * x) - ex), gy = hmax(0.0f, expf(-a * y * y) - ey);
      return gx * gy;
    }
    case BLING_FILTER_MITCHELL: {
      float w = fp[0], h = fp[1], b = fp[2], c = fp[3];
      float iw = 1.0f / w, ih = 1.0f / h;
      auto m1d = [&](float xp) {
        float xx = fabsf(2.0f * xp);
        if (xx > 1)
          return (((-b) - 6.0f * c) * xx * xx * xx + (6.0f * b + 30.0f * c) * xx * xx +
                  ((-12.0f) * b - 48.0f * c) * xx + (8.0f * b + 24.0f * c)) *
                 (1.0f / 6.0f);
        return ((12.0f - 9.0f * b - 6.0f * c) * xx * xx * xx +
                ((-18.0f) + 12.0f * b + 6.0f * c) * xx * xx + (6.0f - 2.0f * b)) *
               (1.0f / 6.0f);
      };
      return m1d(x * iw) * m1d(y * ih);
    }
    case BLING_FILTER_SINC: {
      float ix = 1.0f / fp[0], iy = 1.0f / fp[1], tau = fp[2];
      auto s1 = [&](float xx) {
        if (fabsf(xx) > 1) return 0.0f;
        if (fabsf(xx) < 1e-5f) return 1.0f;
        float xp = fabsf(xx) * kPi;
        float lanczos = sinf(xp * tau) / (xp * tau);
        float sinc = sinf(xp) / xp;
        return sinc * lanczos;
      };
      return s1(x * ix) * s1(y * iy);
    }
    case BLING_FILTER_TRIANGLE: {
      float w = fp[0], h = fp[1];
      float v = hmax(0.0f, w - fabsf(x * 2.0f)) * hmax(0.0f, h - fabsf(y * 2.0f));
      return v / (w * h);
    }
    default: return (fabsf(x) < 0.5f && fabsf(y) < 0.5f) ? 1.0f : 0.0f;
  }
}

template <class T>
cudaError_t devAlloc(T** p, size_t count) {
  return cudaMalloc((void**)p, count * sizeof(T));
}

bool g_const_ready[64] = {false};

cudaError_t ensureConstants(int device) {
  if (device >= 0 && device < 64 && g_const_ready[device]) return cudaSuccess;
  float x[16], y[16], z[16];
  for (int i = 0; i < 16; i++) {
    x[i] = fbits(BLING_CIE_X_BITS[i]);
    y[i] = fbits(BLING_CIE_Y_BITS[i]);
    z[i] = fbits(BLING_CIE_Z_BITS[i]);
  }
  float ys = fbits(BLING_CIE_Y_SUM_BITS);
  cudaError_t e;
  if ((e = cudaMemcpyToSymbol(c_cieX, x, sizeof x)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_cieY, y, sizeof y)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_cieZ, z, sizeof z)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_cieYSum, &ys, sizeof ys)) != cudaSuccess) return e;
  if (device >= 0 && device < 64) g_const_ready[device] = true;
  return cudaSuccess;
}

// sY on the host (for the environment map's importance distribution)
float sYHost(const float* s) {
  float acc = 0.0f;
  for (int i = 0; i < 16; i++) acc = acc + s[i] * fbits(BLING_CIE_Y_BITS[i]);
  return acc / fbits(BLING_CIE_Y_SUM_BITS);
}
// mkDist1D (Montecarlo.hs:269-277)
void mkDist1D(const float* func, int n, float* cdf, float& fi) {
  std::vector<float> i(n + 1);
  i[0] = 0;
  for (int k = 0; k < n; k++) i[k + 1] = i[k] + func[k] / (float)n;
  fi = i[n];
  for (int k = 0; k <= n; k++) cdf[k] = fi != 0 ? i[k] / fi : (float)k / (float)n;
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

int integrator_upload_scene(cudaStream_t stream, const bling_scene_desc& d,
                            const std::vector<int32_t>& order, const std::vector<int32_t>& prim_owner,
                            const std::vector<int32_t>& prim_tri, const std::vector<DShape>& shapes,
                            const std::vector<int32_t>& shape_light, std::vector<void*>& owned,
                            DevShading& out, std::string& err) {
  out = DevShading{};
  size_t bytes = 0;
  auto up = [&](const void* host, size_t nbytes, void** dptr) -> int {
    *dptr = nullptr;
    if (nbytes == 0) return BLING_OK;
    RET_CUDA(cudaMalloc(dptr, nbytes));
    owned.push_back(*dptr);
    bytes += nbytes;
    RET_CUDA(cudaMemcpyAsync(*dptr, host, nbytes, cudaMemcpyHostToDevice, stream));
    return BLING_OK;
  };
  int rc;
  // materials
  std::vector<DMaterial> mats(d.n_materials);
  for (int i = 0; i < d.n_materials; i++) {
    const bling_material& m = d.materials[i];
    DMaterial& o = mats[i];
    o.kind = m.kind;
    o.sigma = m.sigma;
    o.rough = m.roughness;
    o.ior = m.ior;
    memcpy(o.kd, m.kd, 64);
    memcpy(o.ks, m.ks, 64);
    memcpy(o.kt, m.kt, 64);
    memcpy(o.eta, m.eta, 64);
    memcpy(o.k, m.k, 64);
  }
  void* dm;
  if ((rc = up(mats.data(), mats.size() * sizeof(DMaterial), &dm))) return rc;
  out.materials = (const DMaterial*)dm;
  out.n_materials = d.n_materials;
  // meshes
  std::vector<DMesh> meshes(d.n_meshes);
  for (int i = 0; i < d.n_meshes; i++) {
    const bling_mesh_desc& m = d.meshes[i];
    DMesh& o = meshes[i];
    memset(&o, 0, sizeof o);
    void* p;
    if ((rc = up(m.vertices, (size_t)m.n_vertices * 12, &p))) return rc;
    o.verts = (const float*)p;
    if ((rc = up(m.indices, (size_t)m.n_indices * 4, &p))) return rc;
    o.idx = (const int32_t*)p;
    if (m.normals) {
      if ((rc = up(m.normals, (size_t)m.n_vertices * 12, &p))) return rc;
      o.normals = (const float*)p;
    }
    if (m.uvs) {
      if ((rc = up(m.uvs, (size_t)m.n_vertices * 8, &p))) return rc;
      o.uvs = (const float*)p;
    }
    o.material = m.material;
  }
  void* dmesh;
  if ((rc = up(meshes.data(), meshes.size() * sizeof(DMesh), &dmesh))) return rc;
  out.meshes = (const DMesh*)dmesh;
  // per-primitive owner
  std::vector<int2> info(prim_owner.size());
  for (size_t i = 0; i < info.size(); i++) info[i] = make_int2(prim_owner[i], prim_tri[i]);
  void* dinfo;
  if ((rc = up(info.data(), info.size() * sizeof(int2), &dinfo))) return rc;
  out.prim_info = (const int2*)dinfo;
  // shape emission
  std::vector<float> em(16 * std::max<size_t>(1, d.n_shapes), 0.0f);
  for (int i = 0; i < d.n_shapes; i++) memcpy(&em[16 * i], d.shapes[i].emission, 64);
  void* dem;
  if ((rc = up(em.data(), em.size() * 4, &dem))) return rc;
  out.shape_emission = (const float*)dem;
  // lights: the non-geometric ones, then the emissive shapes in primitive order
  std::vector<DLight> lights;
  for (int i = 0; i < d.n_lights; i++) {
    const bling_light_desc& l = d.lights[i];
    DLight o;
    memset(&o, 0, sizeof o);
    o.kind = l.kind;
    o.shape = -1;
    memcpy(o.spec, l.spectrum, 64);
    memcpy(o.vec, l.vec, 12);
    memcpy(o.w2l, l.w2l, 64);
    memcpy(o.l2w, l.l2w, 64);
    if (l.kind == BLING_LIGHT_INFINITE) {
      int w = l.env_w, h = l.env_h;
      if (w <= 0 || h <= 0 || !l.env) {
        err = "infinite light without an environment map";
        return BLING_ERR_INVALID_ARG;
      }
      o.env_w = w;
      o.env_h = h;
      void* p;
      if ((rc = up(l.env, (size_t)w * h * 64, &p))) return rc;
      o.env = (const float*)p;
      // mkInfiniteAreaLight's Dist2D over sY of each texel (Light.hs:76-82,
      // Montecarlo.hs:309-317)
      std::vector<float> func((size_t)w * h), cdf((size_t)h * (w + 1)), cint(h), mcdf(h + 1);
      for (int v = 0; v < h; v++) {
        for (int u = 0; u < w; u++) {
          float uu = (float)u / (float)w, vv = (float)v / (float)h;
          int x = std::max(0, std::min(w - 1, (int)floorf(uu * (float)w)));
          int y = std::max(0, std::min(h - 1, (int)floorf(vv * (float)h)));
          func[(size_t)v * w + u] = sYHost(l.env + 16 * ((size_t)y * w + x));
        }
        mkDist1D(&func[(size_t)v * w], w, &cdf[(size_t)v * (w + 1)], cint[v]);
      }
      float mint;
      mkDist1D(cint.data(), h, mcdf.data(), mint);
      if ((rc = up(func.data(), func.size() * 4, &p))) return rc;
      o.cond_func = (const float*)p;
      if ((rc = up(cdf.data(), cdf.size() * 4, &p))) return rc;
      o.cond_cdf = (const float*)p;
      if ((rc = up(cint.data(), cint.size() * 4, &p))) return rc;
      o.cond_int = (const float*)p;
      if ((rc = up(mcdf.data(), mcdf.size() * 4, &p))) return rc;
      o.marg_cdf = (const float*)p;
      o.marg_int = mint;
    }
    lights.push_back(o);
  }
  for (int32_t v : order) {
    if (v >= 0 || shape_light[~v] < 0) continue;
    DLight o;
    memset(&o, 0, sizeof o);
    o.kind = DLIGHT_AREA;
    o.shape = ~v;
    lights.push_back(o);
  }
  void* dl;
  if ((rc = up(lights.data(), lights.size() * sizeof(DLight), &dl))) return rc;
  out.lights = (const DLight*)dl;
  out.n_lights = (int32_t)lights.size();
  out.camera = d.camera;
  out.bytes = bytes;
  (void)shapes;
  return BLING_OK;
}

void integrator_workspace_free(IntegratorWorkspace& ws) {
  cudaFree(ws.T);
  cudaFree(ws.L);
  cudaFree(ws.ray);
  cudaFree(ws.hit_t);
  cudaFree(ws.hit_prim);
  cudaFree(ws.hit_b);
  cudaFree(ws.queue[0]);
  cudaFree(ws.queue[1]);
  cudaFree(ws.counters);
  cudaFree(ws.filter);
  ws = IntegratorWorkspace{};
}

static int ensureWorkspace(IntegratorWorkspace& ws, size_t cap, std::string& err) {
  if (ws.capacity >= cap && ws.counters) return BLING_OK;
  integrator_workspace_free(ws);
  RET_CUDA(devAlloc(&ws.T, 16 * cap));
  RET_CUDA(devAlloc(&ws.L, 16 * cap));
  RET_CUDA(devAlloc(&ws.ray, 7 * cap));
  RET_CUDA(devAlloc(&ws.hit_t, cap));
  RET_CUDA(devAlloc(&ws.hit_prim, cap));
  RET_CUDA(devAlloc(&ws.hit_b, 2 * cap));
  RET_CUDA(devAlloc(&ws.queue[0], cap));
  RET_CUDA(devAlloc(&ws.queue[1], cap));
  RET_CUDA(devAlloc(&ws.counters, 8));
  RET_CUDA(devAlloc(&ws.filter, 256));
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
  // imageWindow' (Image.hs:170-176)
  P.x0 = (int)floorf(0.5f - fwid);
  P.x1 = (int)floorf(0.5f + (float)p.width + fwid);
  P.y0 = (int)floorf(0.5f - fhei);
  P.y1 = (int)floorf(0.5f + (float)p.height + fhei);
  P.nx = P.x1 - P.x0 + 1;
  P.ny = P.y1 - P.y0 + 1;
  P.nu = p.strata_x;
  P.nv = p.strata_y;
  P.spp = p.strata_x * p.strata_y;
  P.n1d = 4 * p.sample_depth;  // Path.hs:34-36
  P.n2d = 3 * p.sample_depth;
  P.max_depth = p.max_depth;
  P.rr_depth = p.rr_depth;
  P.width = fw;
  P.height = fh;
  uint64_t total = (uint64_t)P.nx * P.ny * P.spp;
  if (total >= (uint64_t(1) << 40)) {
    err = "too many samples in one pass";
    return BLING_ERR_INVALID_ARG;
  }
  // filter table (mkTableFilter, Image.hs:48-61)
  float tbl[256];
  for (int y = 0; y < 16; y++) {
    float fy = ((float)y + 0.5f) * fhei / 16.0f;
    for (int x = 0; x < 16; x++) {
      float fx = ((float)x + 0.5f) * fwid / 16.0f;
      tbl[y * 16 + x] = evalFilterHost(p.filter_kind, p.filter_params, fx, fy);
    }
  }
  RET_CUDA(cudaMemcpyToSymbolAsync(c_filter, tbl, sizeof tbl, 0, cudaMemcpyHostToDevice, stream));
  size_t cap = (size_t)std::min<uint64_t>(total, uint64_t(1) << 22);
  int rc = ensureWorkspace(ws, std::max<size_t>(cap, 1024), err);
  if (rc) return rc;
  RET_CUDA(cudaMemsetAsync(ws.counters, 0, 8 * sizeof(unsigned long long), stream));
  Slots st{ws.T, ws.L, ws.ray, ws.hit_t, ws.hit_prim, ws.hit_b, ws.capacity};
  int sms = 0;
  RET_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int block = 128;
  unsigned grid_full = (unsigned)std::max(1, sms * 8);
  for (uint64_t base = 0; base < total; base += ws.capacity) {
    int64_t count = (int64_t)std::min<uint64_t>(ws.capacity, total - base);
    P.chunk_base = base;
    unsigned g = (unsigned)std::min<int64_t>((count + block - 1) / block, grid_full);
    k_raygen<<<g, block, 0, stream>>>(P, S.camera, st, count, ws.queue[0], ws.counters);
    RET_CUDA(cudaGetLastError());
    for (int depth = 0; depth <= p.max_depth; depth++) {
      int in = depth & 1;
      RET_CUDA(cudaMemsetAsync(ws.counters + 5, 0, sizeof(unsigned long long), stream));
      k_trace<<<std::min(g, traceGrid(sms)), block, 0, stream>>>(A, st, ws.queue[in],
                                                                 ws.counters + in, ws.counters);
      RET_CUDA(cudaGetLastError());
      k_reset_count<<<1, 1, 0, stream>>>(ws.counters + (1 - in));
      k_shade<<<g, block, 0, stream>>>(A, S, P, st, depth, ws.queue[in], ws.counters + in,
                                        ws.queue[1 - in], ws.counters + (1 - in), d_film,
                                        ws.counters);
      RET_CUDA(cudaGetLastError());
    }
  }
  unsigned long long cnt[8];
  RET_CUDA(cudaMemcpyAsync(cnt, ws.counters, sizeof cnt, cudaMemcpyDeviceToHost, stream));
  RET_CUDA(cudaStreamSynchronize(stream));
  res.rays_closest = cnt[2];
  res.rays_any = cnt[3];
  res.nonfinite = cnt[4];
  res.path_samples = total;
  return BLING_OK;
}

// ------------------------------------------------------------------ no-allocation pass
// Path state for bling_render_pass_noalloc, in one file-scope device array:
// the wavefront of one pass of at most kNoAllocSlots path samples.  Every GPU
// that loads the library holds these 11.5 MiB (plus 64 bytes of counters)
// until the process exits.  All calls share the array; the counters are
// cleared at the start of every call, the path state is written before it is
// read.  Two calls whose work overlaps on the GPU (different streams or
// contexts on one device) race on it.
constexpr size_t kNoAllocSlots = size_t(1) << 16;
// per slot: T (16 f), L (16 f), ray (7 f), hit t (1 f), hit prim (1 i),
// hit barycentrics (2 f), two queue entries (2 i)
constexpr size_t kNoAllocWordsPerSlot = 16 + 16 + 7 + 1 + 1 + 2 + 2;
constexpr size_t kNoAllocCounterBytes = 256;
constexpr size_t kNoAllocBytes = kNoAllocCounterBytes + kNoAllocWordsPerSlot * 4 * kNoAllocSlots;
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
  for (int y = 0; y < 16; y++) {
    float fy = ((float)y + 0.5f) * fhei / 16.0f;
    for (int x = 0; x < 16; x++) {
      float fx = ((float)x + 0.5f) * fwid / 16.0f;
      tbl[y * 16 + x] = evalFilterHost(p.filter_kind, p.filter_params, fx, fy);
    }
  }
  RET_CUDA(cudaMemcpyToSymbolAsync(c_filter, tbl, sizeof tbl, 0, cudaMemcpyHostToDevice, stream));
  // carve the path state out of the array
  const size_t cap = kNoAllocSlots;
  unsigned char* base = g_noalloc_ptr[device];
  unsigned long long* counters = (unsigned long long*)base;
  float* words = (float*)(base + kNoAllocCounterBytes);
  Slots st{words, words + 16 * cap, words + 32 * cap, words + 39 * cap,
           (int32_t*)(words + 40 * cap), words + 41 * cap, cap};
  int32_t* queue[2] = {(int32_t*)(words + 43 * cap), (int32_t*)(words + 44 * cap)};
  RET_CUDA(cudaMemsetAsync(counters, 0, 8 * sizeof(unsigned long long), stream));
  int sms = 0;
  RET_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int block = 128;
  int64_t count = (int64_t)total;
  P.chunk_base = 0;
  unsigned g = (unsigned)std::min<int64_t>((count + block - 1) / block, std::max(1, sms * 8));
  k_raygen<<<g, block, 0, stream>>>(P, S.camera, st, count, queue[0], counters);
  RET_CUDA(cudaGetLastError());
  for (int depth = 0; depth <= p.max_depth; depth++) {
    int in = depth & 1;
    RET_CUDA(cudaMemsetAsync(counters + 5, 0, sizeof(unsigned long long), stream));
    k_trace<<<std::min(g, traceGrid(sms)), block, 0, stream>>>(A, st, queue[in], counters + in,
                                                               counters);
    RET_CUDA(cudaGetLastError());
    k_reset_count<<<1, 1, 0, stream>>>(counters + (1 - in));
    k_shade<<<g, block, 0, stream>>>(A, S, P, st, depth, queue[in], counters + in, queue[1 - in],
                                      counters + (1 - in), d_film, counters);
    RET_CUDA(cudaGetLastError());
  }
  unsigned long long cnt[8];
  RET_CUDA(cudaMemcpyAsync(cnt, counters, sizeof cnt, cudaMemcpyDeviceToHost, stream));
  RET_CUDA(cudaStreamSynchronize(stream));
  res.rays_closest = cnt[2];
  res.rays_any = cnt[3];
  res.nonfinite = cnt[4];
  res.path_samples = total;
  return BLING_OK;
}

}  // namespace bgpu
