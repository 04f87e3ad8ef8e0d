// Device helpers of the wavefront path integrator: spectra, the sampler and
// its counter-based generator, Monte Carlo warps, BSDFs and materials, hit
// geometry, lights and the film splat.  Each restates the reference function it
// names (src/lib/Graphics/Bling/...).  Every translation unit that includes it
// is built with -fmad=false so the arithmetic rounds like the reference's
// binary32, and has its own copy of the constant tables below.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>
#include <mutex>

#include "dmath.cuh"
#include "dshape.cuh"
#include "integrator.h"
#include "spectrum_tables.h"
#include "texture.cuh"
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
__device__ __forceinline__ Spec sLoad(const float* p) {  // p in global memory
  Spec s;
#pragma unroll
  for (int i = 0; i < 16; i++) s.v[i] = __ldg(p + i);
  return s;
}
// a material spectrum a BxDF points at: the scene's record in global memory,
// or a textured material resolved into the shading thread's local memory,
// so generic loads rather than the read-only global path
__device__ __forceinline__ Spec sLoadAny(const float* p) {
  Spec s;
#pragma unroll
  for (int i = 0; i < 16; i++) s.v[i] = p[i];
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
__device__ __forceinline__ bool allFinite(const Spec& s) {
  bool b = true;
#pragma unroll
  for (int i = 0; i < 16; i++) b = b && isfinite(s.v[i]);
  return b;
}
__device__ __forceinline__ Spec sClamp01(const Spec& a) {
  Spec s;
#pragma unroll
  for (int i = 0; i < 16; i++) s.v[i] = hmax(0.0f, hmin(1.0f, a.v[i]));
  return s;
}

static __constant__ float c_cieX[16], c_cieY[16], c_cieZ[16];
static __constant__ float c_cieYSum;

// fills this translation unit's CIE tables on the current device (once per
// device; callers on several threads serialise on a mutex)
static cudaError_t loadCieConstants(int device) {
  static std::mutex mu;
  static bool ready[64] = {false};
  std::lock_guard<std::mutex> g(mu);
  if (device >= 0 && device < 64 && ready[device]) return cudaSuccess;
  auto bits = [](uint32_t b) {
    float f;
    memcpy(&f, &b, 4);
    return f;
  };
  float x[16], y[16], z[16];
  for (int i = 0; i < 16; i++) {
    x[i] = bits(BLING_CIE_X_BITS[i]);
    y[i] = bits(BLING_CIE_Y_BITS[i]);
    z[i] = bits(BLING_CIE_Z_BITS[i]);
  }
  float ys = bits(BLING_CIE_Y_SUM_BITS);
  cudaError_t e;
  if ((e = cudaMemcpyToSymbol(c_cieX, x, sizeof x)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_cieY, y, sizeof y)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_cieZ, z, sizeof z)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_cieYSum, &ys, sizeof ys)) != cudaSuccess) return e;
  if (device >= 0 && device < 64) ready[device] = true;
  return cudaSuccess;
}

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
  int random;  // Random sampler (Sampling.hs:101-110): no strata, fresh uniforms
  uint64_t chunk_base;
};

// ------------------------------------------------------------------ Monte Carlo
// concentricSampleDisk (Montecarlo.hs:160-179)
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

enum { BX_LAMBERT, BX_OREN, BX_SPEC_REFL, BX_SPEC_TRANS, BX_MICRO, BX_FBLEND };
enum { T_REFL = 1, T_TRANS = 2, T_DIFF = 4, T_GLOSSY = 8, T_SPEC = 16 };
enum { FR_NOOP, FR_DIEL, FR_COND };

struct BxDF {
  int kind, type;
  const float* r;  // spectrum of the material (global or local memory), null = white
  float A, B;      // Oren-Nayar
  float ei, et;    // dielectric Fresnel / transmission
  float e;         // Blinn exponent
  int fr;
  const float* eta;
  const float* k;
  bool clampR;     // glass: sClamp' of the colour
  bool btdf;       // brdfToBtdf (Reflection.hs:188-195): wi in the other hemisphere
};
__device__ __forceinline__ V3 otherHemisphere(V3 w) { return V3{w.x, w.y, -w.z}; }
__device__ __forceinline__ Spec bxR(const BxDF& b) {
  if (!b.r) return sConst(1.0f);
  Spec s = sLoadAny(b.r);
  return b.clampR ? sClamp01(s) : s;
}

// frDielectric (Fresnel.hs:21-56), one value for all bands
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
  // frConductor (Fresnel.hs:58-70)
  float acosi = fabsf(cosi);
  Spec out;
#pragma unroll
  for (int i = 0; i < 16; i++) {
    float eta = b.eta[i], k = b.k[i];
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

// the Anisotropic microfacet distribution (Microfacet.hs:136-192): ex, ey
__device__ __forceinline__ float anisoPdf(float ex, float ey, V3 wh) {
  float costh = absCosTheta(wh);
  float e = (ex * wh.x * wh.x + ey * wh.y * wh.y) / hmax(0.0f, 1.0f - costh * costh);
  return sqrtf((ex + 1.0f) * (ey + 1.0f)) * kInvTwoPi * powf(costh, e);
}
__device__ __forceinline__ float anisoD(float ex, float ey, V3 wh) {
  float costh = absCosTheta(wh);
  float d = 1.0f - costh * costh;
  if (d == 0) return 0;
  float e = (ex * wh.x * wh.x + ey * wh.y * wh.y) / d;
  return sqrtf((ex + 2.0f) * (ey + 2.0f)) * kInvTwoPi * powf(costh, e);
}
__device__ __forceinline__ void anisoSample(float ex, float ey, float u1, float u2, V3& wh,
                                            float& pdf) {
  float phi, cost;
  auto quad = [&](float up, int which) {
    float p = ex == ey ? kPi * up * 0.5f : atanf(sqrtf((ex + 1.0f) / (ey + 1.0f)) * tanf(kPi * up * 0.5f));
    float cp = cosf(p), sp = sinf(p);
    cost = powf(u2, 1.0f / (ex * cp * cp + ey * sp * sp + 1.0f));
    phi = which == 0 ? p : (which == 1 ? kPi - p : (which == 2 ? p + kPi : 2.0f * kPi - p));
  };
  if (u1 < 0.25f)
    quad(4.0f * u1, 0);
  else if (u1 < 0.5f)
    quad(4.0f * (0.5f - u1), 1);
  else if (u1 < 0.75f)
    quad(4.0f * (u1 - 0.5f), 2);
  else
    quad(4.0f * (1.0f - u1), 3);
  float sint = sqrtf(hmax(0.0f, 1.0f - cost * cost));
  wh = V3{sint * cosf(phi), sint * sinf(phi), cost};
  float ds = 1.0f - cost * cost;
  float e = (ex * wh.x * wh.x + ey * wh.y * wh.y) / ds;
  float f = kInvTwoPi * powf(cost, e);
  pdf = sqrtf((ex + 1.0f) * (ey + 1.0f)) * f;
}
// FresnelBlend's e wo wi (Microfacet.hs:63-86): rd in r, rs in eta, ra in k,
// the distribution's exponents in A and B, the coating depth in e
__device__ __forceinline__ Spec fblendEval(const BxDF& b, V3 wo, V3 wi) {
  float costi = absCosTheta(wi), costo = absCosTheta(wo);
  Spec rd = sLoadAny(b.r), rs = sLoadAny(b.eta), ra = sLoadAny(b.k);
  Spec a = sConst(1.0f);
  if (b.e > 0) {
    float x = -(b.e * (costi + costo) / (costi * costo));
#pragma unroll
    for (int i = 0; i < 16; i++) a.v[i] = expf(ra.v[i] * x);
  }
  float ds = ((costo * 28.0f / 23.0f) * kPi) * (1.0f - powf(1.0f - 0.5f * costi, 5.0f)) *
             (1.0f - powf(1.0f - 0.5f * costo, 5.0f));
  Spec diff = sScale(a * rd * (sConst(1.0f) - rs), ds);
  V3 wh = normalize(wi + wo);
  if (wh.z < 0) wh = -wh;
  float costih = absDot(wi, wh);
  Spec schlick = rs + sScale(sConst(1.0f) - rs, powf(1.0f - costih, 5.0f));
  Spec spec = sScale(schlick, anisoD(b.A, b.B, wh) * costo / (4.0f * costih * hmax(costi, costo)));
  return diff + spec;
}

// bxdfEval b wo wi
// Inlining of the BSDF, geometry and light helpers below is left to the
// compiler: keeping them out of line (__noinline__) measured 18% slower in
// the shading kernel, whose instruction-fetch stalls come from divergence
// between materials rather than from code size.
#define BLING_OUTLINE

static __device__ BLING_OUTLINE Spec bxEval(const BxDF& b, V3 wo, V3 wi) {
  if (b.btdf) wi = otherHemisphere(wi);
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
    case BX_FBLEND: return fblendEval(b, wo, wi);
    default: return sConst(0);
  }
}
// the BRDF's pdf (a BTDF's sample calls its BRDF's sample, Reflection.hs:192-193)
static __device__ BLING_OUTLINE float bxPdfBrdf(const BxDF& b, V3 wo, V3 wi) {
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
    case BX_FBLEND: {  // Microfacet.hs:104-108
      if (!sameHemisphere(wo, wi)) return 0;
      V3 wh = normalize(wi + wo);
      if (wh.z < 0) wh = -wh;
      return 0.5f * (absCosTheta(wi) * kInvPi + anisoPdf(b.A, b.B, wh) / (4.0f * absDot(wo, wh)));
    }
    default: return 0;
  }
}
static __device__ BLING_OUTLINE float bxPdf(const BxDF& b, V3 wo, V3 wi) {
  return bxPdfBrdf(b, wo, b.btdf ? otherHemisphere(wi) : wi);
}
// bxdfSample b Adj wo u (Diffuse.hs:14-49, Specular.hs:12-58,
// Microfacet.hs:42-54); Adj = the adjoint transport of light paths
template <bool Adj>
static __device__ BLING_OUTLINE void bxSampleBrdf(const BxDF& b, V3 wo, float u1, float u2, Spec& f, V3& wi, float& pdf);
template <bool Adj = false>
static __device__ BLING_OUTLINE void bxSample(const BxDF& b, V3 wo, float u1, float u2, Spec& f, V3& wi, float& pdf) {
  bxSampleBrdf<Adj>(b, wo, u1, u2, f, wi, pdf);
  if (b.btdf) wi = otherHemisphere(wi);
}
template <bool Adj>
static __device__ BLING_OUTLINE void bxSampleBrdf(const BxDF& b, V3 wo, float u1, float u2, Spec& f, V3& wi, float& pdf) {
  switch (b.kind) {
    case BX_LAMBERT:
    case BX_OREN: {
      wi = toSameHemisphere(wo, cosineSampleHemisphere(u1, u2));
      if (sameHemisphere(wo, wi)) {
        f = b.kind == BX_LAMBERT ? bxR(b) : sScale(bxR(b), orenNayarScale(b, wo, wi));
        if (Adj) f = sScale(f, fabsf(cosTheta(wo) / cosTheta(wi)));
        pdf = bxPdfBrdf(b, wo, wi);
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
    case BX_FBLEND: {  // Microfacet.hs:88-102
      V3 wh;
      float pdfp;
      if (u1 < 0.5f) {
        wi = toSameHemisphere(wo, cosineSampleHemisphere(u1 * 2.0f, u2));
        wh = normalize(wi + wo);
        if (wh.z < 0) wh = -wh;
        pdfp = anisoPdf(b.A, b.B, wh);
      } else {
        anisoSample(b.A, b.B, 2.0f * (u1 - 0.5f), u2, wh, pdfp);
        wi = sv(2.0f * dot(wo, wh), wh) - wo;
      }
      if (pdfp == 0) {
        f = sConst(0);
        pdf = 0;
        return;
      }
      pdf = 0.5f * (absCosTheta(wi) * kInvPi + pdfp / (4.0f * absDot(wo, wh)));
      f = sScale(Adj ? fblendEval(b, wi, wo) : fblendEval(b, wo, wi), 1.0f / pdf);
      return;
    }
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
      float fr = frDielScalar(ei, et, Adj ? cosTheta(wo) : cost);
      Spec t = bxR(b);
      float sc = Adj ? fabsf(cosTheta(wo) / cost) : eta2;
#pragma unroll
      for (int i = 0; i < 16; i++) f.v[i] = ((1.0f - fr) * t.v[i]) * sc;
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
        f = sScale(rTimesFresnel(b, costH), fact / absCosTheta(Adj ? wo : wi));
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

// mkBsdf' with the material's BxDFs (Material.hs:32-127).  The Bsdf keeps
// pointers into m, which must outlive it.
static __device__ BLING_OUTLINE Bsdf materialBsdf(const DMaterial& m, V3 dgg_n, V3 dgs_p, V3 dgs_n,
                                                  V3 dgs_dpdu) {
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
  x.btdf = false;
  int kind = m.kind;
  float sigma = m.sigma, rough = m.rough, ior = m.ior;
  // the kd texture at the shading point
  const float* kd = m.kd;
  if (m.kd_tex == BLING_TEX_CHECKER) {  // checkerBoard (Texture.hs:209-219)
    long long c = (long long)floorf(dgs_p.x * m.kd_par[0]) + (long long)floorf(dgs_p.y * m.kd_par[1]) +
                  (long long)floorf(dgs_p.z * m.kd_par[2]);
    if (c % 2 != 0) kd = m.kd2;  // Haskell's mod 2 is 0 for even sums of either sign
  } else if (m.kd_tex == BLING_TEX_GRAPH_PAPER) {  // graphPaper + planarMapping (Texture.hs:172-207)
    const float* q = m.kd_par;
    float u = dot(dgs_p, V3{q[1], q[2], q[3]}) + q[7], v = dot(dgs_p, V3{q[4], q[5], q[6]}) + q[8];
    float xf = fabsf(u - truncf(u)), zf = fabsf(v - truncf(v));  // properFraction
    float lo = q[0] / 2.0f, hi = 1.0f - lo;
    if (xf < lo || zf < lo || xf > hi || zf > hi) kd = m.kd2;
  }
  if (kind == BLING_MAT_MATTE) {
    x.type = T_REFL | T_DIFF;
    x.r = kd;
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
    x.r = kd;
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
  } else if (kind == BLING_MAT_SHINY_METAL) {
    // mkShinyMetal (Material.hs:98-109): a Blinn microfacet lobe and a
    // specular one, both white, with conductor Fresnel terms approximated
    // from ks and kr (derived at upload into eta/k and kd/kt)
    x.kind = BX_MICRO;
    x.type = T_REFL | T_GLOSSY;
    x.e = fixExponent(1.0f / rough);
    x.fr = FR_COND;
    x.eta = m.eta;
    x.k = m.k;
    b.c[b.n++] = x;
    BxDF y = x;
    y.kind = BX_SPEC_REFL;
    y.type = T_REFL | T_SPEC;
    y.e = 0;
    y.eta = m.kd;
    y.k = m.kt;
    b.c[b.n++] = y;
  } else if (kind == BLING_MAT_TRANS_MATTE) {
    // translucentMatte (Material.hs:43-53): Lambertian or Oren-Nayar
    // reflection of r and the same lobe of t turned into a BTDF (r and t
    // derived at upload into kd and kt)
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
    BxDF y = x;
    y.type = T_TRANS | T_DIFF;
    y.r = m.kt;
    y.btdf = true;
    b.c[b.n++] = y;
  } else if (kind == BLING_MAT_SUBSTRATE) {
    // mkSubstrate (Material.hs:111-127): one FresnelBlend lobe; the clamped
    // spectra and the anisotropic exponents are derived at upload
    x.kind = BX_FBLEND;
    x.type = T_REFL | T_GLOSSY;
    x.r = kd;
    x.eta = m.ks;
    x.k = m.kt;
    x.A = m.rough;
    x.B = m.sigma;
    x.e = m.ior;
    b.c[b.n++] = x;
  } else if (kind == BLING_MAT_BLACKBODY) {
    // blackBodyMaterial (Reflection.hs:337-338): no BxDFs
  } else if (kind == BLING_MAT_MIRROR) {
    // mirrorMaterial: specRefl frNoOp (sClamp 0 1 kr) (Material.hs:68-72)
    x.kind = BX_SPEC_REFL;
    x.type = T_REFL | T_SPEC;
    x.r = m.ks;
    x.clampR = true;
    x.fr = FR_NOOP;
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

// sampleBsdf'' Adj bxdfAll (Reflection.hs:278-316); Adj = sampleAdjBsdf
template <bool Adj = false>
static __device__ BLING_OUTLINE BsdfSample sampleBsdf(const Bsdf& b, V3 woW, float uComp, float u1, float u2) {
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
  bxSample<Adj>(bx, wo, u1, u2, fSample, wi, pdfp);
  V3 wiW = localToWorld(b.cs, wi);
  float sideTest = dot(wiW, b.ng) / dot(woW, b.ng);
  if (pdfp == 0 || sideTest == 0) return out;
  bool wantTrans = sideTest < 0;
  bool ok = wantTrans ? (bx.type & T_TRANS) != 0 : (bx.type & T_REFL) != 0;
  if (!ok) return out;
  out.type = bx.type;
  out.wi = wiW;
  // fAdj: the adjoint's correction for shading normals
  const float adjScale = fabsf(sideTest);
  if (bx.type & T_SPEC) {
    out.pdf = pdfp * invCnt;
    out.f = sScale(Adj ? sScale(fSample, adjScale) : fSample, cntf);
    return out;
  }
  if (cntm == 1) {
    out.pdf = pdfp;
    out.f = Adj ? sScale(fSample, adjScale) : fSample;
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
    if (ok2) fOthers = fOthers + (Adj ? bxEval(b.c[i], wo, wi) : bxEval(b.c[i], wi, wo));
  }
  out.pdf = pdf;
  out.f = sScale(sScale(fSample, pdfp) + fOthers, 1.0f / pdf);
  if (Adj) out.f = sScale(out.f, adjScale);
  return out;
}
// bsdfHasNonSpecular (Reflection.hs:246-249)
__device__ __forceinline__ bool bsdfHasNonSpecular(const Bsdf& b) {
  for (int i = 0; i < b.n; i++)
    if (!(b.c[i].type & T_SPEC)) return true;
  return false;
}
// sampleBsdf'' False flags (Reflection.hs:278-316) over the BxDFs whose type
// lies within `flags` (bxdfMatches, Reflection.hs:119-121, 185-186)
static __device__ BsdfSample sampleBsdfFlags(const Bsdf& b, V3 woW, int flags, float uComp,
                                             float u1, float u2) {
  BsdfSample out;
  out.type = T_REFL | T_DIFF;
  out.pdf = 0;
  out.f = sConst(0);
  out.wi = V3{0, 1, 0};
  int idx[2], cntm = 0;
  for (int i = 0; i < b.n; i++)
    if ((b.c[i].type & flags) == b.c[i].type) idx[cntm++] = i;
  if (cntm == 0) return out;
  V3 wo = worldToLocal(b.cs, woW);
  float cntf = (float)cntm;
  float invCnt = 1.0f / cntf;
  int sNum = max(0, min(cntm - 1, (int)floorf(uComp * cntf)));
  const BxDF& bx = b.c[idx[sNum]];
  Spec fSample;
  V3 wi;
  float pdfp;
  bxSample<false>(bx, wo, u1, u2, fSample, wi, pdfp);
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
  for (int j = 0; j < cntm; j++)
    if (j != sNum) others = others + bxPdf(b.c[idx[j]], wo, wi);
  float pdf = (pdfp + others) * invCnt;
  Spec fOthers = sConst(0);
  for (int j = 0; j < cntm; j++) {
    if (j == sNum) continue;
    const BxDF& o = b.c[idx[j]];
    bool ok2 = wantTrans ? (o.type & T_TRANS) != 0 : (o.type & T_REFL) != 0;
    if (ok2) fOthers = fOthers + bxEval(o, wi, wo);
  }
  out.pdf = pdf;
  out.f = sScale(sScale(fSample, pdfp) + fOthers, 1.0f / pdf);
  return out;
}
// evalBsdf Adj (Reflection.hs:318-332)
template <bool Adj = false>
static __device__ BLING_OUTLINE Spec evalBsdf(const Bsdf& b, V3 woW, V3 wiW) {
  float cosWo = dot(woW, b.ng);
  float sideTest = dot(wiW, b.ng) / cosWo;
  if (sideTest == 0) return sConst(0);
  if (fabsf(cosWo) < 1e-5f) return sConst(0);
  bool wantTrans = sideTest < 0;
  V3 wo = worldToLocal(b.cs, woW), wi = worldToLocal(b.cs, wiW);
  Spec f = sConst(0);
  for (int i = 0; i < b.n; i++) {
    bool ok = wantTrans ? (b.c[i].type & T_TRANS) != 0 : (b.c[i].type & T_REFL) != 0;
    if (ok) f = f + (Adj ? bxEval(b.c[i], wo, wi) : bxEval(b.c[i], wi, wo));
  }
  return Adj ? sScale(f, fabsf(sideTest)) : f;  // shading-normal correction of the adjoint
}
// bsdfPdf (Reflection.hs:251-257)
static __device__ BLING_OUTLINE float bsdfPdf(const Bsdf& b, V3 woW, V3 wiW) {
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
// the rest of the shading geometry that textured materials read: surface
// parameters and the derivatives bump mapping tilts
struct TexFrame {
  float u, v;
  V3 sdpdv, dndu, dndv;
};

template <bool FRAME>
static __device__ __forceinline__ HitGeom hitGeometryT(const DevAccel& A, const DevShading& S,
                                                       const Ray& r, int prim, float t, float b1,
                                                       float b2, TexFrame* tf) {
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
    // transDg o2w (DifferentialGeometry.hs:71-81)
    g.p = transPoint(sh.o2w, dg.p);
    g.n = normalize(transNormal(sh.w2o, dg.n));
    g.sdpdu = transVector(sh.o2w, dg.dpdu);
    if (FRAME) {
      tf->sdpdv = transVector(sh.o2w, dg.dpdv);
      tf->dndu = transNormal(sh.w2o, dg.dndu);
      tf->dndv = transNormal(sh.w2o, dg.dndv);
      tf->u = dg.u;
      tf->v = dg.v;
    }
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
  if (FRAME) {  // the interpolated (u, v) (TriangleMesh.hs:198-201); dndu = dndv = 0
    float b0 = 1.0f - b1 - b2;
    tf->u = b0 * uv00 + b1 * uv10 + b2 * uv20;
    tf->v = b0 * uv01 + b1 * uv11 + b2 * uv21;
    tf->sdpdv = dpdv;
    tf->dndu = tf->dndv = V3{0, 0, 0};
  }
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
    V3 ss, ts;
    if (sqLen(tsp) > 0) {
      ts = normalize(tsp);
      ss = cross(ts, ns);
    } else {
      LC c = coordinateSystem(ns);
      ss = c.s;
      ts = c.t;
    }
    g.sn = ns;
    g.sdpdu = ss;
    if (FRAME) tf->sdpdv = ts;
  }
  return g;
}
static __device__ BLING_OUTLINE HitGeom hitGeometry(const DevAccel& A, const DevShading& S,
                                                    const Ray& r, int prim, float t, float b1,
                                                    float b2) {
  return hitGeometryT<false>(A, S, r, prim, t, b1, b2, nullptr);
}
static __device__ BLING_OUTLINE void hitTexFrame(const DevAccel& A, const DevShading& S,
                                                 const Ray& r, int prim, float t, float b1,
                                                 float b2, TexFrame& tf) {
  hitGeometryT<true>(A, S, r, prim, t, b1, b2, &tf);
}

// ------------------------------------------------------------------ textured materials
// bump d dgg dgs (Reflection.hs:347-377): the displacement at the shading
// point and one hundredth of a step along u and along v tilts dpdu and dpdv
// along the shading normal; the new normal is turned to the side of the
// geometric one.  (The shifted points' normals do not enter: textures read
// only p, u and v.)
static __device__ void bumpShading(const DTex* T, int d, const TexFrame& f, HitGeom& g) {
  const float du = 0.01f, dv = 0.01f;
  TexGeo gs{g.sp, f.u, f.v};
  TexGeo geu{g.sp + sv(du, g.sdpdu), f.u + du, f.v};
  TexGeo gev{g.sp + sv(dv, f.sdpdv), f.u, f.v + dv};
  float uDisp = texScalar(T, d, geu), vDisp = texScalar(T, d, gev), disp = texScalar(T, d, gs);
  float vscale = (vDisp - disp) / dv;
  V3 dpdv = f.sdpdv + sv(vscale, g.sn);
  float uscale = (uDisp - disp) / du;
  V3 dpdu = g.sdpdu + sv(uscale, g.sn);
  V3 nn = normalize(cross(dpdu, dpdv));
  if (dot(nn, g.n) < 0) nn = -nn;  // faceForward nn' (dgN dgg)
  g.sn = nn;
  g.sdpdu = dpdu;
}

// material mi with its textures evaluated at tg (Material.hs: every texture
// takes dgs) and its derived spectra made, in `scratch`
static __device__ __noinline__ const DMaterial* texturedMaterial(const DevShading& S, int mi,
                                                                  const TexGeo& tg,
                                                                  DMaterial& scratch) {
  const DMaterial& m = S.materials[mi];
  scratch = m;
  float* spectra[5] = {scratch.kd, scratch.ks, scratch.kt, scratch.eta, scratch.k};
  for (int slot = 0; slot < 5; slot++)
    if (m.tex[slot]) texSpectrum(S.tex, m.tex[slot] - 1, tg, spectra[slot]);
  if (m.tex[0]) scratch.kd_tex = BLING_TEX_CONSTANT;
  if (m.tex[5]) scratch.sigma = texScalar(S.tex, m.tex[5] - 1, tg);
  if (m.tex[6]) scratch.rough = texScalar(S.tex, m.tex[6] - 1, tg);
  if (m.tex[7]) scratch.ior = texScalar(S.tex, m.tex[7] - 1, tg);
  deriveMaterialSpectra(scratch);
  return &scratch;
}

// A textured material at hit g (prim hit by r at t, b1, b2): the bump tilts
// g's shading frame, the textures are evaluated at the hit, the result goes
// to `scratch`; uv, if given, receives the hit's (u, v).  Kept out of line:
// the kernels that shade pay only for the test in hitMaterial.
static __device__ __noinline__ const DMaterial* resolveTextured(const DevAccel& A,
                                                                const DevShading& S, const Ray& r,
                                                                int prim, float t, float b1,
                                                                float b2, HitGeom& g,
                                                                DMaterial& scratch, float* uv) {
  const DMaterial& m = S.materials[g.material];
  TexFrame f;
  hitTexFrame(A, S, r, prim, t, b1, b2, f);
  if (uv) {
    uv[0] = f.u;
    uv[1] = f.v;
  }
  if (m.bump) bumpShading(S.tex, m.bump - 1, f, g);
  return texturedMaterial(S, g.material, TexGeo{g.sp, f.u, f.v}, scratch);
}
// The material of hit g: the scene's record, or for a textured material
// (bumpMapped, or parameters that name texture nodes) its resolution at the
// hit in `scratch`.
__device__ __forceinline__ const DMaterial* hitMaterial(const DevAccel& A, const DevShading& S,
                                                        const Ray& r, int prim, float t, float b1,
                                                        float b2, HitGeom& g, DMaterial& scratch,
                                                        float* uv = nullptr) {
  const DMaterial* m = S.materials + g.material;
  if (!m->textured) return m;
  return resolveTextured(A, S, r, prim, t, b1, b2, g, scratch, uv);
}

// ------------------------------------------------------------------ lights
__device__ __forceinline__ bool insideSphere(float r, V3 p) { return sqLen(p) - r * r < 1e-4f; }

static __device__ void sampleShapeP(const DShape& s, float u1, float u2, V3& p, V3& n) {
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
static __device__ BLING_OUTLINE void sampleShape(const DShape& s, V3 pt, float u1, float u2, V3& ps, V3& ns) {
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
static __device__ BLING_OUTLINE float shapePdf(const DShape& s, V3 p, V3 wi) {
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
// texMapEval of an infinite light's map at (u, v): the texel of an image
// map (getPixel, Texture.hs:96-101), or the sun/sky model at (u, v)
static __device__ BLING_OUTLINE Spec envEval(const DLight& l, float u, float v) {
  if (l.sky) {
    Spec s;
    skyEval(*l.sky, u, v, s.v);
    return s;
  }
  return sLoad(envTexel(l, u, v));
}
// upperBound + sampleContinuous1D (Montecarlo.hs:53-73); findIndex (>= u)
// on a non-decreasing CDF is its lower bound
static __device__ void sampleContinuous1D(const float* func, const float* cdf, int n, float fi, float u,
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

static __device__ BLING_OUTLINE LightSample lightSample(const DevAccel& A, const DevShading& S, const DLight& l, V3 p,
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
  // infinite (Light.hs:130-141), sampleContinuous2D (Montecarlo.hs:90-93)
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
  ls.li = envEval(l, u, v);
  V3 dl{sinf(theta) * cosf(phi), sinf(theta) * sinf(phi), cosf(theta)};
  ls.wi = transVector(l.l2w, dl);
  ls.ray = Ray{p, ls.wi, eps, INFINITY};
  ls.pdf = mapPdf / (2.0f * kPi * kPi * sint);
  return ls;
}
// le (Light.hs:98-106)
static __device__ BLING_OUTLINE Spec lightLe(const DLight& l, V3 d) {
  if (l.kind != DLIGHT_INFINITE) return sConst(0);
  V3 wh = normalize(transVector(l.w2l, d));
  float phi = sphericalPhi(wh), theta = sphericalTheta(wh);
  return envEval(l, phi / (2.0f * kPi), theta / kPi);
}
// pdf (Light.hs:215-229)
static __device__ BLING_OUTLINE float lightPdf(const DevAccel& A, const DLight& l, V3 p, V3 wi) {
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
// the pass's 16x16 filter table in device memory (the caller's workspace), so
// passes of different contexts on one device never share it
struct TableFilter {
  const float* t;
  __device__ __forceinline__ float operator()(int i) const { return __ldg(t + i); }
};

// addSample (Image.hs:250-299) into the tile image of the sample's tile
// (mkImageTile/addTile, Image.hs:108-120,178-199): the footprint is clipped to
// the tile's pixel range and to the film.  filt(i) reads entry i of the 16x16
// filter table.
// Returns false when the sample is dropped as NaN/Inf.
template <class Filter>
__device__ bool filmAddT(float* __restrict__ film, const PassParams& P, int ix, int iy, float sx,
                         float sy, const Spec& L, unsigned long long* nonfinite, Filter filt) {
  bool bad = false;
#pragma unroll
  for (int i = 0; i < 16; i++) bad = bad || isnan(L.v[i]) || isinf(L.v[i]);
  if (bad) {
    atomicAdd(nonfinite, 1ull);
    return false;
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
      float w = filt(iyf * 16 + ixf);
      float* px = film + 4 * ((size_t)y * P.width + x);
      atomicAdd(px, w);
      atomicAdd(px + 1, smx * w);
      atomicAdd(px + 2, smy * w);
      atomicAdd(px + 3, smz * w);
    }
  }
  return true;
}

}  // namespace bgpu
