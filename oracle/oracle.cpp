// CPU oracle for the GB300 path-tracing core of bling.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, function by function, the
// reference's Haskell code for the hot path (file:line citations are to the
// reference, src/lib/Graphics/Bling/...).  It is the parity checker for the
// GPU library and the timed host-core baseline; the product never links it.
//
// Arithmetic: IEEE binary32, one rounding per operation in the reference's
// order, no contraction (built with -ffp-contract=off).  Transcendentals call
// the C library's float functions, as GHC's Float primops do.
//
// Randomness: the reference draws from mwc-random seeded from system entropy
// per tile (Rendering.hs:128, Random.hs:61-62, 91-96), a stream that cannot be
// reproduced.  The oracle and the GPU therefore share one counter-based
// generator (SplitMix64 finaliser, Steele/Lea/Flood 2014) keyed by
// (seed, pass, pixel, sample, dimension), and the stratified sample
// dimensions use Kensler's hash permutation (Correlated Multi-Jittered
// Sampling, 2013) in place of the reference's in-place shuffles
// (Sampling.hs:134-152).  The sample structure -- which dimensions are
// stratified, jittered and shuffled -- follows the reference.
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

#include "../bling_gb300/csrc/spectrum_tables.h"
#include "kdtree.h"
#include "oracle_math.h"

using namespace orc;

namespace {

// ---------------------------------------------------------------- spectra
// Spectrum.hs:33-46: 16 bands
struct Spec {
  float v[16];
};
static inline Spec sConst(float c) {
  Spec s;
  for (int i = 0; i < 16; i++) s.v[i] = c;
  return s;
}
static const Spec BLACK = sConst(0.0f);
static const Spec WHITE = sConst(1.0f);
static inline Spec operator+(const Spec& a, const Spec& b) {
  Spec s;
  for (int i = 0; i < 16; i++) s.v[i] = a.v[i] + b.v[i];
  return s;
}
static inline Spec operator-(const Spec& a, const Spec& b) {
  Spec s;
  for (int i = 0; i < 16; i++) s.v[i] = a.v[i] - b.v[i];
  return s;
}
static inline Spec operator*(const Spec& a, const Spec& b) {
  Spec s;
  for (int i = 0; i < 16; i++) s.v[i] = a.v[i] * b.v[i];
  return s;
}
static inline Spec operator/(const Spec& a, const Spec& b) {
  Spec s;
  for (int i = 0; i < 16; i++) s.v[i] = a.v[i] / b.v[i];
  return s;
}
// sScale (Spectrum.hs:448-450)
static inline Spec sScale(const Spec& a, float f) {
  Spec s;
  for (int i = 0; i < 16; i++) s.v[i] = a.v[i] * f;
  return s;
}
static inline bool isBlack(const Spec& s) {
  for (int i = 0; i < 16; i++)
    if (s.v[i] != 0) return false;
  return true;
}
static inline bool sNaN(const Spec& s) {
  for (int i = 0; i < 16; i++)
    if (std::isnan(s.v[i])) return true;
  return false;
}
static inline bool sInf(const Spec& s) {
  for (int i = 0; i < 16; i++)
    if (std::isinf(s.v[i])) return true;
  return false;
}
static inline Spec sClamp(float lo, float hi, const Spec& a) {
  Spec s;
  for (int i = 0; i < 16; i++) s.v[i] = hmax(lo, hmin(hi, a.v[i]));
  return s;
}
static inline float tbl(const uint32_t* bits, int i) { return __bling_f32(bits[i]); }

// sY (Spectrum.hs:371-373)
static float sY(const Spec& s) {
  float acc = 0.0f;
  for (int i = 0; i < 16; i++) acc = acc + s.v[i] * tbl(BLING_CIE_Y_BITS, i);
  return acc / __bling_f32(BLING_CIE_Y_SUM_BITS);
}
// spectrumToXYZ (Spectrum.hs:349-355)
static void spectrumToXYZ(const Spec& s, float& x, float& y, float& z) {
  float a = 0, b = 0, c = 0;
  for (int i = 0; i < 16; i++) {
    float v = s.v[i];
    a = a + tbl(BLING_CIE_X_BITS, i) * v;
    b = b + tbl(BLING_CIE_Y_BITS, i) * v;
    c = c + tbl(BLING_CIE_Z_BITS, i) * v;
  }
  float ys = __bling_f32(BLING_CIE_Y_SUM_BITS);
  x = a / ys;
  y = b / ys;
  z = c / ys;
}
// rgbToSpectrum (Spectrum.hs:146-159)
static Spec basis(bool illum, int which) {
  Spec s;
  const uint32_t* t = illum ? BLING_RGB_ILLUM_BITS : BLING_RGB_REFL_BITS;
  for (int i = 0; i < 16; i++) s.v[i] = tbl(t, which * 16 + i);
  return s;
}
static Spec rgbToSpectrum(bool illum, float r, float g, float b) {
  Spec wb = basis(illum, BLING_BASIS_WHITE), cb = basis(illum, BLING_BASIS_CYAN),
       mb = basis(illum, BLING_BASIS_MAGENTA), yb = basis(illum, BLING_BASIS_YELLOW),
       rb = basis(illum, BLING_BASIS_RED), gb = basis(illum, BLING_BASIS_GREEN),
       bb = basis(illum, BLING_BASIS_BLUE);
  if (r <= g && r <= b) {
    return sScale(wb, r) + (g <= b ? sScale(cb, g - r) + sScale(bb, b - g)
                                   : sScale(cb, b - r) + sScale(gb, g - b));
  }
  if (g <= r && g <= b) {
    return sScale(wb, g) + (r <= b ? sScale(mb, r - g) + sScale(bb, b - r)
                                   : sScale(mb, b - g) + sScale(rb, r - b));
  }
  return sScale(wb, b) + (r <= b ? sScale(yb, r - b) + sScale(gb, g - r)
                                 : sScale(yb, g - b) + sScale(rb, r - g));
}
// xyzToRgb (Spectrum.hs:162-168)
static void xyzToRgb(float x, float y, float z, float& r, float& g, float& b) {
  r = 3.240479f * x - 1.537150f * y - 0.498535f * z;
  g = (-0.969256f) * x + 1.875991f * y + 0.041556f * z;
  b = 0.055648f * x - 0.204043f * y + 1.057311f * z;
}

// ---------------------------------------------------------------- randomness
static inline uint64_t mix64(uint64_t z) {
  z ^= z >> 30;
  z *= 0xbf58476d1ce4e5b9ULL;
  z ^= z >> 27;
  z *= 0x94d049bb133111ebULL;
  z ^= z >> 31;
  return z;
}
static inline uint64_t pixelKey(uint64_t seed, uint64_t pass, int px, int py) {
  uint64_t k = mix64(seed ^ mix64(pass + 0x9e3779b97f4a7c15ULL));
  return mix64(k ^ (((uint64_t)(uint32_t)px << 32) | (uint64_t)(uint32_t)py));
}
static inline uint32_t randU32(uint64_t key, uint32_t n, uint32_t dim) {
  return (uint32_t)(mix64(key ^ mix64(((uint64_t)n << 32) | dim)) >> 32);
}
static inline float randF(uint64_t key, uint32_t n, uint32_t dim) {
  return (float)(randU32(key, n, dim) >> 8) * (1.0f / 16777216.0f);
}
// Kensler's permute(i, l, p): a hashed bijection on [0, l)
static uint32_t permute(uint32_t i, uint32_t l, uint32_t p) {
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

// dimension ids of the shared generator
enum : uint32_t {
  DIM_PIX_U = 0,
  DIM_PIX_V = 1,
  DIM_LENS_PERM = 2,
  DIM_LENS_U = 3,
  DIM_LENS_V = 4,
  DIM_1D_BASE = 16,        // + 2*off (perm), + 2*off + 1 (jitter)
  DIM_2D_BASE = 4096,      // + 4*off (perm), +1 (ju), +2 (jv)
  DIM_FRESH_1D = 1u << 20, // | n
  DIM_FRESH_2D = 2u << 20  // | 2n + {0,1}
};
static const float ALMOST_ONE = 0.9999999403953552f;  // Sampling.hs:154-155

// One camera sample of the stratified sampler (Sampling.hs:112-132, 157-171)
struct Sampler {
  uint64_t key;
  uint32_t n;       // sample index within the pixel
  int nu, nv;       // strata
  int n1d, n2d;     // precomputed dimension counts
};
// stratified2D entry i: (u, v) = quotRem i nu (Sampling.hs:164-171)
static void strat2D(const Sampler& s, uint32_t i, uint32_t dju, uint32_t djv, float& u, float& v) {
  float du = 1.0f / (float)s.nu, dv = 1.0f / (float)s.nv;
  uint32_t qu = i / (uint32_t)s.nu, qv = i % (uint32_t)s.nu;
  float ju = randF(s.key, i, dju), jv = randF(s.key, i, djv);
  u = hmin(ALMOST_ONE, ((float)qu + ju) * du);
  v = hmin(ALMOST_ONE, ((float)qv + jv) * dv);
}
// rnd' n (Sampling.hs:203-211)
static float rnd1(const Sampler& s, int n) {
  if (n < s.n1d) {
    uint32_t N = (uint32_t)(s.nu * s.nv);
    uint32_t p = randU32(s.key, 0xffffffffu, DIM_1D_BASE + 2 * n);
    uint32_t st = permute(s.n, N, p);
    float du = 1.0f / (float)N;
    float j = randF(s.key, st, DIM_1D_BASE + 2 * n + 1);
    return hmin(ALMOST_ONE, ((float)st + j) * du);
  }
  return randF(s.key, s.n, DIM_FRESH_1D | (uint32_t)n);
}
// rnd2D' n (Sampling.hs:213-221)
static void rnd2(const Sampler& s, int n, float& u, float& v) {
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

// ---------------------------------------------------------------- geometry
struct DG {  // DifferentialGeometry (DifferentialGeometry.hs:26-36)
  V p, n;
  float u, v;
  V dpdu, dpdv, dndu, dndv;
  bool tri;
  float b1, b2;
};
// mkDg: n = normalize (dpdu x dpdv) (DifferentialGeometry.hs:41-51)
static DG mkDg(V p, float u, float v, V dpdu, V dpdv, V dndu, V dndv) {
  DG g;
  g.p = p;
  g.n = normalize(cross(dpdu, dpdv));
  g.u = u;
  g.v = v;
  g.dpdu = dpdu;
  g.dpdv = dpdv;
  g.dndu = dndu;
  g.dndv = dndv;
  g.tri = false;
  g.b1 = g.b2 = 0;
  return g;
}
// mkDg' p n: dpdu/dpdv from coordinateSystem n (DifferentialGeometry.hs:53-56)
static DG mkDg2(V p, V n) {
  LC c = coordinateSystem(n);
  DG g;
  g.p = p;
  g.n = n;
  g.u = g.v = 0;
  g.dpdu = c.s;
  g.dpdv = c.t;
  g.dndu = g.dndv = V{0, 0, 0};
  g.tri = false;
  g.b1 = g.b2 = 0;
  return g;
}
// transDg (DifferentialGeometry.hs:72-81)
static DG transDg(const float* m, const float* mi, const DG& g) {
  DG r = g;
  r.p = transPoint(m, g.p);
  r.n = normalize(transNormal(mi, g.n));
  r.dpdu = transVector(m, g.dpdu);
  r.dpdv = transVector(m, g.dpdv);
  r.dndu = transNormal(mi, g.dndu);
  r.dndv = transNormal(mi, g.dndv);
  return r;
}

// solveQuadric (Math.hs:124-139)
static bool solveQuadric(float a, float b, float c, float& t0, float& t1) {
  float discrim = b * b - 4.0f * a * c;
  if (discrim < 0) return false;
  float rootDiscrim = sqrtf(discrim);
  float q = b < 0 ? -0.5f * (b - rootDiscrim) : -0.5f * (b + rootDiscrim);
  float x0 = q / a, x1 = c / q;
  t0 = hmin(x0, x1);
  t1 = hmax(x0, x1);
  return true;
}

// intersectAABB (AABB.hs:79-94)
static bool intersectAABB(V bmin, V bmax, const Ray& r, float& n_out, float& f_out) {
  float near = r.tmin, far = r.tmax;
  for (int dim = 0; dim < 3; dim++) {
    if (near > far) return false;
    float dInv = 1.0f / comp(r.d, dim);
    float oc = comp(r.o, dim);
    float tFar = (comp(bmax, dim) - oc) * dInv;
    float tNear = (comp(bmin, dim) - oc) * dInv;
    float nn = tNear > tFar ? tFar : tNear, ff = tNear > tFar ? tNear : tFar;
    near = hmax(near, nn);
    far = hmin(far, ff);
  }
  if (near > far) return false;
  n_out = near;
  f_out = far;
  return true;
}

struct Shape {
  int kind;
  float p[6];
  Xf o2w;  // m = o2w, i = w2o
  int material;
  bool emissive;
  Spec emission;
  int light_id;  // index into the scene's light list when emissive
};

// area (Shape.hs:314-328)
static float shapeArea(const Shape& s) {
  switch (s.kind) {
    case BLING_SHAPE_BOX: {
      float h = s.p[3] - s.p[0], w = s.p[4] - s.p[1], l = s.p[5] - s.p[2];
      return 2.0f * (h * w + h * l + w * l);
    }
    case BLING_SHAPE_CYLINDER: return 2.0f * PI * s.p[0] * (s.p[2] - s.p[1]);
    case BLING_SHAPE_DISK: {
      float rmin2 = s.p[2] * s.p[2], rmax2 = s.p[1] * s.p[1];
      return PI * (rmax2 - rmin2);
    }
    case BLING_SHAPE_QUAD: return 4.0f * s.p[0] * s.p[1];
    default: return s.p[0] * s.p[0] * 4.0f * PI;
  }
}

// Shape.intersect in object space (Shape.hs:81-229); returns t, eps, dg
static bool shapeIntersect(const Shape& s, const Ray& ray, float& t_out, float& e_out, DG& dg) {
  const V& ro = ray.o;
  const V& rd = ray.d;
  float tmin = ray.tmin, tmax = ray.tmax;
  switch (s.kind) {
    case BLING_SHAPE_BOX: {
      V pmin{s.p[0], s.p[1], s.p[2]}, pmax{s.p[3], s.p[4], s.p[5]};
      float near = -INF, far = INF;
      int dd = 0;
      for (int dim = 0; dim < 3; dim++) {
        if (near > far) return false;
        float dInv = 1.0f / comp(rd, dim);
        float oc = comp(ro, dim);
        float t1p = (comp(pmax, dim) - oc) * dInv;
        float t2p = (comp(pmin, dim) - oc) * dInv;
        float t1 = t1p > t2p ? t2p : t1p, t2 = t1p > t2p ? t1p : t2p;
        int ndd = near < t1 ? dim : dd;
        near = hmax(near, t1);
        far = hmin(far, t2);
        dd = ndd;
      }
      if (near > far) return false;
      float t0 = hmin(near, far), t1 = hmax(near, far);
      if (t0 > tmax || t0 < tmin) return false;
      float t = t0 < tmin ? t1 : t0;
      if (t > tmax) return false;
      V p = rayAt(ray, t);
      float half = (comp(pmin, dd) + comp(pmax, dd)) / 2.0f;
      float dir = comp(p, dd) > half ? 1.0f : -1.0f;
      V n = normalize(setComp(dd, dir, mkV(0, 0, 0)));
      t_out = t;
      e_out = 5e-4f * t;
      dg = mkDg2(p, n);
      return true;
    }
    case BLING_SHAPE_CYLINDER: {
      float r = s.p[0], zmin = s.p[1], zmax = s.p[2], phimax = s.p[3];
      float a = rd.x * rd.x + rd.y * rd.y;
      float b = 2.0f * (rd.x * ro.x + rd.y * ro.y);
      float c = ro.x * ro.x + ro.y * ro.y - r * r;
      float t0, t1;
      if (!solveQuadric(a, b, c, t0, t1)) return false;
      if (t0 > tmax) return false;
      if (t1 < tmin) return false;
      V ph0 = rayAt(ray, t0), ph1 = rayAt(ray, t1);
      float phi0 = atan2p(ph0.y, ph0.x), phi1 = atan2p(ph1.y, ph1.x);
      V ph;
      float t;
      if (t0 > tmin && ph0.z > zmin && ph0.z < zmax && phi0 <= phimax) {
        ph = ph0;
        t = t0;
      } else if (t1 <= tmax && ph1.z > zmin && ph1.z < zmax && phi1 <= phimax) {
        ph = ph1;
        t = t1;
      } else {
        return false;
      }
      V dpdu{-phimax * ph.y, phimax * ph.x, 0};
      V dpdv{0, 0, zmax - zmin};
      t_out = t;
      e_out = 5e-4f * t;
      dg = mkDg2(ph, normalize(cross(dpdu, dpdv)));
      return true;
    }
    case BLING_SHAPE_DISK: {
      float h = s.p[0], rad = s.p[1], irad = s.p[2], phimax = s.p[3];
      if (fabsf(rd.z) < 1e-7f) return false;
      float t = (h - ro.z) / rd.z;
      if (t < tmin || t > tmax) return false;
      V p = rayAt(ray, t);
      float d2 = p.x * p.x + p.y * p.y;
      if (d2 > rad * rad || d2 < irad * irad) return false;
      float phi = atan2p(p.y, p.x);
      if (phi > phimax) return false;
      t_out = t;
      e_out = 5e-4f * t;
      dg = mkDg2(p, mkV(0, 0, -1));
      return true;
    }
    case BLING_SHAPE_QUAD: {
      float sx = s.p[0], sy = s.p[1];
      if (fabsf(rd.z) < 1e-7f) return false;
      float t = -(ro.z) / rd.z;
      if (t < tmin || t > tmax) return false;
      V p = rayAt(ray, t);
      if (fabsf(p.x) > sx || fabsf(p.y) > sy) return false;
      t_out = t;
      e_out = 5e-4f * t;
      // u = (sx + px) / (2 sx), v = (sy + py) / (2 sy) (Shape.hs:164-171)
      dg = mkDg(p, (sx + p.x) / (2.0f * sx), (sy + p.y) / (2.0f * sy), mkV(sx, 0, 0),
                mkV(0, sy, 0), V{0, 0, 0}, V{0, 0, 0});
      return true;
    }
    default: {  // sphere
      float r = s.p[0];
      float a = sqLen(rd);
      float b = 2.0f * dot(ro, rd);
      float c = sqLen(ro) - r * r;
      float t1, t2;
      if (!solveQuadric(a, b, c, t1, t2)) return false;
      if (t1 > tmax) return false;
      if (t2 < tmin) return false;
      float t = t1 < tmin ? t2 : t1;
      if (t > tmax) return false;
      V p = rayAt(ray, t);
      const float thetaMax = 0.0f, thetaMin = PI, phiMax = TWO_PI;
      float theta = acosf(clampf(p.z / r, -1, 1));
      float zradius = sqrtf(p.x * p.x + p.y * p.y);
      float invz = 1.0f / zradius;
      float cosphi = p.x * invz, sinphi = p.y * invz;
      V dpdu{-phiMax * p.y, phiMax * p.x, 0};
      V dpdv = V{p.z * cosphi, p.z * sinphi, -r * sinf(theta)} * V{thetaMax - thetaMin,
                                                                 thetaMax - thetaMin,
                                                                 thetaMax - thetaMin};
      float phi = atan2p(p.y, p.x);
      float u = phi / phiMax, v = (theta - thetaMin) / (thetaMax - thetaMin);
      // dndu, dndv from the fundamental forms (Shape.hs:209-229)
      float kk = thetaMax - thetaMin;
      auto vp = [](float x) { return V{x, x, x}; };  // vpromote
      V d2Pduu = vp(-phiMax * phiMax) * mkV(p.x, p.y, 0);
      V d2Pduv = vp(kk * p.z * phiMax) * mkV(-sinphi, cosphi, 0);
      V d2Pdvv = vp(-kk * kk) * mkV(p.x, p.y, p.z);
      float e1 = dot(dpdu, dpdu), f1 = dot(dpdu, dpdv), g1 = dot(dpdv, dpdv);
      V n1 = normalize(cross(dpdu, dpdv));
      float e = dot(n1, d2Pduu), f = dot(n1, d2Pduv), g = dot(n1, d2Pdvv);
      float invEGF2 = 1.0f / (e1 * g1 - f1 * f1);
      V dndu = vp((f * f1 - e * g1) * invEGF2) * dpdu + vp((e * f1 - f * e1) * invEGF2) * dpdv;
      V dndv = vp((g * f1 - f * g1) * invEGF2) * dpdu + vp((f * f1 - g * e1) * invEGF2) * dpdv;
      t_out = t;
      e_out = 5e-4f * t;
      dg = mkDg(p, u, v, dpdu, dpdv, dndu, dndv);
      return true;
    }
  }
}

// Shape.intersects in object space (Shape.hs:231-284)
static bool shapeIntersects(const Shape& s, const Ray& ray) {
  const V& ro = ray.o;
  const V& rd = ray.d;
  float tmin = ray.tmin, tmax = ray.tmax;
  switch (s.kind) {
    case BLING_SHAPE_BOX: {
      float n, f;
      return intersectAABB(V{s.p[0], s.p[1], s.p[2]}, V{s.p[3], s.p[4], s.p[5]}, ray, n, f);
    }
    case BLING_SHAPE_CYLINDER: {
      float r = s.p[0], zmin = s.p[1], zmax = s.p[2], phimax = s.p[3];
      float a = rd.x * rd.x + rd.y * rd.y;
      float b = 2.0f * (rd.x * ro.x + rd.y * ro.y);
      float c = ro.x * ro.x + ro.y * ro.y - r * r;
      float t0, t1;
      if (!solveQuadric(a, b, c, t0, t1)) return false;
      if (t0 > tmax) return false;
      if (t1 < tmin) return false;
      V ph0 = rayAt(ray, t0), ph1 = rayAt(ray, t1);
      float phi0 = atan2p(ph0.y, ph0.x), phi1 = atan2p(ph1.y, ph1.x);
      if (t0 > tmin && ph0.z > zmin && ph0.z < zmax && phi0 <= phimax) return true;
      if (t1 < tmax && ph1.z > zmin && ph1.z < zmax && phi1 <= phimax && t1 <= tmax) return true;
      return false;
    }
    case BLING_SHAPE_DISK: {
      float h = s.p[0], rad = s.p[1], irad = s.p[2], phimax = s.p[3];
      if (fabsf(rd.z) < 1e-7f) return false;
      float t = (h - ro.z) / rd.z;
      if (t < tmin || t > tmax) return false;
      V p = rayAt(ray, t);
      float d2 = p.x * p.x + p.y * p.y;
      if (d2 > rad * rad || d2 < irad * irad) return false;
      return !(atan2p(p.y, p.x) > phimax);
    }
    case BLING_SHAPE_QUAD: {
      if (fabsf(rd.z) < 1e-7f) return false;
      float t = -(ro.z) / rd.z;
      if (t < tmin || t > tmax) return false;
      V p = rayAt(ray, t);
      return !(fabsf(p.x) > s.p[0] || fabsf(p.y) > s.p[1]);
    }
    default: {
      float r = s.p[0];
      float a = sqLen(rd);
      float b = 2.0f * dot(ro, rd);
      float c = sqLen(ro) - r * r;
      float t0, t1;
      if (!solveQuadric(a, b, c, t0, t1)) return false;
      if (t0 > tmax || t1 < tmin) return false;
      if (t0 < tmin) return t1 < tmax;
      return true;
    }
  }
}

// ---------------------------------------------------------------- scene
struct Mesh {
  std::vector<V> p;
  std::vector<int32_t> idx;
  std::vector<V> n;       // empty: no shading normals
  std::vector<float> uv;  // empty: default uvs
  int material;
};

enum BxKind { BX_LAMBERT, BX_OREN, BX_SPEC_REFL, BX_SPEC_TRANS, BX_MICRO, BX_FBLEND };
enum { T_REFL = 1, T_TRANS = 2, T_DIFF = 4, T_GLOSSY = 8, T_SPEC = 16 };
enum FrKind { FR_NOOP, FR_DIEL, FR_COND };

struct Fresnel {
  int kind;
  float ei, et;    // dielectric
  Spec eta, k;     // conductor
};

struct BxDF {
  int kind;
  int type;
  Spec r;
  float A, B;       // Oren-Nayar
  float ei, et;     // specular transmission
  float e;          // Blinn exponent
  Fresnel fr;
  bool btdf;        // brdfToBtdf (Reflection.hs:188-195)
  Spec rs, ra;      // FresnelBlend: specular, absorption (rd in r; ex, ey in A, B; depth in e)
};
static inline V otherHemisphere(V w) { return V{w.x, w.y, -w.z}; }

struct Material {
  int kind;
  float sigma, rough, ior;
  Spec kd, ks, kt, eta, k;
  int kd_tex;
  float kd_par[9];
  Spec kd2;
  int tex[8];  // texture node + 1 per parameter slot (bling_material.tex)
  int bump;    // displacement node + 1
};

// a texture expression node (bling_texture)
struct TexNode {
  int kind, a, b, c, ivalue, map_kind;
  float map[16], p[4];
  Spec spectrum;
  std::vector<float> steps;    // gradient: (position, spectrum) x ivalue, sorted by position
  std::vector<uint8_t> pixels;  // image
  int w, h;
};

struct Prim {
  int is_shape;
  int index;  // mesh triangle: mesh id; shape: shape id
  int tri;    // triangle number within the mesh
  V p1, p2, p3;
};

// ------------------------------------------------------------ sun and sky
// mkSunSkyLight (SunSky.hs:12-158): the Perez sky plus a solar disc as a
// continuous lat-long map.
struct SkyData {  // SunSky.hs:28-37, plus the disc direction and spectrum
  V sunDir;       // normalize (worldToLocal basis (normalize sunDir))
  V discDir;      // normalize (worldToLocal basis sunDir)
  float sunTheta;
  float perezx[5], perezy[5], perezY[5];
  float zenithx, zenithy, zenithY;
  Spec sunR;
};

// sunThetaMax2 (SunSky.hs:39-43)
static float sunThetaMax2() {
  float sint2 = 6.955e5f / 1.496e8f;
  return sqrtf(hmax(0.0f, 1.0f - sint2));
}

// evalSpd of an IrregularSpd (Spectrum.hs:258-269)
static float spdIrregular(const float* ls, const float* vs, int n, float l) {
  if (l <= ls[0]) return vs[0];
  if (l >= ls[n - 1]) return vs[n - 1];
  int lo = 0, hi = n - 1, i;
  for (;;) {  // fi lo hi
    int mid = (lo + hi) / 2;
    if (lo == mid) {
      i = lo;
      break;
    }
    if (ls[mid] == l) {
      i = mid;
      break;
    }
    if (ls[mid] < l)
      lo = mid;
    else
      hi = mid;
  }
  float t = (l - ls[i]) / (ls[i + 1] - ls[i]);
  return lerp(t, vs[i], vs[i + 1]);
}
// evalSpd of a RegularSpd (Spectrum.hs:271-280)
static float spdRegular(float l0, float l1, const float* amps, int n, float l) {
  if (l <= l0) return amps[0];
  if (l >= l1) return amps[n - 1];
  float d1 = 1.0f / ((l1 - l0) / (float)(n - 1));
  float x = (l - l0) * d1;
  int b0 = (int)std::floor(x);
  int b1 = std::min(b0 + 1, n - 1);
  float dx = x - (float)b0;
  return (1.0f - dx) * amps[b0] + dx * amps[b1];
}

// solCurve, koCurve, kgCurve, kwaCurve (SunSky.hs:127-157)
static const float SOL[] = {165.5f, 162.3f, 211.2f, 258.8f, 258.2f, 242.3f, 267.6f, 296.6f,
                            305.4f, 300.6f, 306.6f, 288.3f, 287.1f, 278.2f, 271.0f, 272.3f,
                            263.6f, 255.0f, 250.6f, 253.1f, 253.5f, 251.3f, 246.3f, 241.7f,
                            236.8f, 232.1f, 228.2f, 223.4f, 219.7f, 215.3f, 211.0f, 207.3f,
                            202.4f, 198.7f, 194.3f, 190.7f, 186.3f, 182.6f};
static const float KO_L[] = {300, 305, 310, 315, 320, 325, 330, 335, 340, 345, 350, 355, 445,
                             450, 455, 460, 465, 470, 475, 480, 485, 490, 495, 500, 505, 510,
                             515, 520, 525, 530, 535, 540, 545, 550, 555, 560, 565, 570, 575,
                             580, 585, 590, 595, 600, 605, 610, 620, 630, 640, 650, 660, 670,
                             680, 690, 700, 710, 720, 730, 740, 750, 760, 770, 780, 790};
static const float KO_A[] = {10.0f,  4.8f,   2.7f,   1.35f,  0.8f,   0.380f, 0.160f, 0.075f,
                             0.04f,  0.019f, 0.007f, 0.0f,   0.003f, 0.003f, 0.004f, 0.006f,
                             0.008f, 0.009f, 0.012f, 0.014f, 0.017f, 0.021f, 0.025f, 0.03f,
                             0.035f, 0.04f,  0.045f, 0.048f, 0.057f, 0.063f, 0.07f,  0.075f,
                             0.08f,  0.085f, 0.095f, 0.103f, 0.110f, 0.12f,  0.122f, 0.12f,
                             0.118f, 0.115f, 0.12f,  0.125f, 0.130f, 0.12f,  0.105f, 0.09f,
                             0.079f, 0.067f, 0.057f, 0.048f, 0.036f, 0.028f, 0.023f, 0.018f,
                             0.014f, 0.011f, 0.010f, 0.009f, 0.007f, 0.004f, 0.0f,   0.0f};
static const float KG_L[] = {759, 760, 770, 771};
static const float KG_A[] = {0.0f, 3.0f, 0.210f, 0.0f};
static const float KWA_L[] = {689, 690, 700, 710, 720, 730, 740, 750, 760, 770, 780, 790, 800};
static const float KWA_A[] = {0.0f,      0.160e-1f, 0.240e-1f, 0.125e-1f, 0.100e+1f,
                              0.870f,    0.610e-1f, 0.100e-2f, 0.100e-4f, 0.100e-4f,
                              0.600e-3f, 0.175e-1f, 0.360e-1f};

// sf of sunSpectrum' (SunSky.hs:102-125)
static float sunSpd(float t, float turb, float l) {
  float m = 1.0f / (cosf(t) + 0.000940f * powf(1.6386f - t, -1.253f));
  float tR = expf(-(m * 0.008735f * powf(l / 1000.0f, -4.08f)));
  float alpha = 1.3f;
  float beta = 0.04608365822050f * turb - 0.04586025928522f;
  float tA = expf(-(m * beta * powf(l / 1000.0f, -alpha)));
  float lozone = 0.35f;
  float tO = expf(-(m * spdIrregular(KO_L, KO_A, 64, l) * lozone));
  float kg = spdIrregular(KG_L, KG_A, 4, l);
  float tG = expf(-(1.41f * kg * m / powf(1.0f + 118.93f * kg * m, 0.45f)));
  float kwa = spdIrregular(KWA_L, KWA_A, 13, l);
  float w = 2.0f;
  float tWA = expf(-(0.2385f * kwa * w * m / powf(1.0f + 20.07f * kwa * w * m, 0.45f)));
  return spdRegular(380.0f, 750.0f, SOL, 38, l) * tR * tA * tO * tG * tWA;
}

// initSky and sunSpectrum' with the basis coordinateSystem' up east
// (SunSky.hs:17-24, 45-65, 96-101; Math.hs:427-441)
static SkyData initSkyData(V east, V sdw, float t) {
  V w = normalize(normalize(mkV(0, 1, 0)));
  V u = normalize(cross(normalize(east), w));
  V v = cross(w, u);
  auto toLocal = [&](V a) { return mkV(dot(a, u), dot(a, v), dot(a, w)); };
  SkyData s;
  s.sunDir = normalize(toLocal(normalize(sdw)));
  s.discDir = normalize(toLocal(sdw));
  float st = acosf(clampf(s.sunDir.z, -1, 1));
  float st2 = st * st, st3 = st * st * st, t2 = t * t;
  float chi = (4.0f / 9.0f - t / 120.0f) * (PI - 2.0f * st);
  s.sunTheta = st;
  const float pY[5] = {0.17872f * t - 1.46303f, -0.35540f * t + 0.42749f,
                       -0.02266f * t + 5.32505f, 0.12064f * t - 2.57705f,
                       -0.06696f * t + 0.37027f};
  const float px[5] = {-0.01925f * t - 0.25922f, -0.06651f * t + 0.00081f,
                       -0.00041f * t + 0.21247f, -0.06409f * t - 0.89887f,
                       -0.00325f * t + 0.04517f};
  const float py[5] = {-0.01669f * t - 0.26078f, -0.09495f * t + 0.00921f,
                       -0.00792f * t + 0.21023f, -0.04405f * t - 1.65369f,
                       -0.01092f * t + 0.05291f};
  for (int i = 0; i < 5; i++) {
    s.perezY[i] = pY[i];
    s.perezx[i] = px[i];
    s.perezy[i] = py[i];
  }
  s.zenithY = ((4.04530f * t - 4.97100f) * tanf(chi) - 0.2155f * t + 2.4192f) * 1000.0f;
  s.zenithx = (0.00165f * st3 - 0.00374f * st2 + 0.00208f * st) * t2 +
              (-0.02902f * st3 + 0.06377f * st2 - 0.03202f * st + 0.00394f) * t +
              (0.11693f * st3 - 0.21196f * st2 + 0.06052f * st + 0.25885f);
  s.zenithy = (0.00275f * st3 - 0.00610f * st2 + 0.00316f * st) * t2 +
              (-0.04212f * st3 + 0.08970f * st2 - 0.04153f * st + 0.00515f) * t +
              (0.15346f * st3 - 0.26756f * st2 + 0.06669f * st + 0.26688f);
  // sunSpectrum': fromSpd (mkSpdFunc sf), each band avgSpd = the mean of the
  // function at the band's two ends (Spectrum.hs:316, 329-335)
  s.sunR = BLACK;
  if (!(s.sunDir.z < 0)) {
    for (int i = 0; i < 16; i++) {
      float l0 = lerp((float)i / 16.0f, 400.0f, 700.0f);
      float l1 = lerp((float)(i + 1) / 16.0f, 400.0f, 700.0f);
      s.sunR.v[i] = (sunSpd(st, t, l0) + sunSpd(st, t, l1)) * 0.5f;
    }
  }
  return s;
}

// perez (SunSky.hs:81-86)
static float perez(const float* p, float sunT, float t, float g, float lvz) {
  float csg = cosf(g), cst = cosf(sunT);
  float num = (1.0f + p[0] * expf(p[1] / cosf(t))) * (1.0f + p[2] * expf(p[3] * g)) + p[4] * csg * csg;
  float den = (1.0f + p[0] * expf(p[1])) * (1.0f + p[2] * expf(p[3] * sunT)) + p[4] * cst * cst;
  return lvz * num / den;
}

// skySpectrum (SunSky.hs:67-79) with chromaticityToXYZ (Spectrum.hs:229-251)
// and xyzToSpectrum (Spectrum.hs:357-358)
static Spec skySpectrum(const SkyData& s, V dir) {
  float dz = -dir.z;
  if (dz < 1e-4f) return BLACK;
  float theta = acosf(dz);
  float gamma = acosf(clampf(dot(dir, s.sunDir), -1, 1));
  float x = perez(s.perezx, s.sunTheta, theta, gamma, s.zenithx);
  float y = perez(s.perezy, s.sunTheta, theta, gamma, s.zenithy);
  float yy = perez(s.perezY, s.sunTheta, theta, gamma, s.zenithY) * 1e-4f;
  float m1 = (-1.3515f - 1.7703f * x + 5.9114f * y) / (0.0241f + 0.2562f * x - 0.7341f * y);
  float m2 = (0.03f - 31.4424f * x + 30.0717f * y) / (0.0241f + 0.2562f * x - 0.7341f * y);
  const uint32_t* S = BLING_CIE_S012_XYZ_BITS;
  float cx = tbl(S, 0) + m1 * tbl(S, 3) + m2 * tbl(S, 6);
  float cy = tbl(S, 1) + m1 * tbl(S, 4) + m2 * tbl(S, 7);
  float cz = tbl(S, 2) + m1 * tbl(S, 5) + m2 * tbl(S, 8);
  float X = cx * yy / cy, Z = cz * yy / cy;
  float r, g, b;
  xyzToRgb(X, yy, Z, r, g, b);
  return rgbToSpectrum(true, r, g, b);
}

// eval of mkSunSkyLight at (u, v): sky plus the disc (SunSky.hs:18-20, 88-94)
static Spec sunSkyEval(const SkyData& s, float u, float v) {
  float phi = u * 2.0f * PI, theta = v * PI;  // cartToSph (Types.hs:31-33)
  V dir = mkV(sinf(theta) * cosf(phi), sinf(theta) * sinf(phi), cosf(theta));  // sphToDir
  Spec r = skySpectrum(s, dir);
  float d = dot(s.discDir * mkV(1, 1, -1), dir);
  return r + (d > sunThetaMax2() ? s.sunR : BLACK);
}

struct Light {
  int kind;  // BLING_LIGHT_* or 100 = area
  Spec spec;
  V vec;
  int shape;  // area lights
  int id;
  // infinite
  std::vector<Spec> env;
  int w, h;
  bool sky;  // the map is mkSunSkyLight's function rather than env
  SkyData skyd;
  Xf w2l;
  // Dist2D (Montecarlo.hs:75-106)
  std::vector<std::vector<float>> cfunc, ccdf;
  std::vector<float> cint;
  std::vector<float> mfunc, mcdf;
  float mint;
};
static const int LIGHT_AREA = 100;

struct AabbF {
  V lo, hi;
};

struct BvhNode {
  double lo[3], hi[3];
  int left, right;  // right < 0: leaf; left = first, -right-1 = count
};

}  // namespace

struct orc_scene {
  std::vector<Mesh> meshes;
  std::vector<Shape> shapes;
  std::vector<Material> mats;
  std::vector<TexNode> tex;
  std::vector<Light> lights;
  std::vector<Prim> prims;
  bling_camera_desc cam;
  // oracle BVH
  std::vector<BvhNode> nodes;
  std::vector<int> order;
  // the reference's kd-tree (kdtree.h), built on request; `use_kd` makes it
  // the accelerator of scIntersect/occluded in the renderers
  kd::Tree kd;
  bool kd_built = false;
  bool use_kd = false;
};

namespace {

// ---------------------------------------------------------------- triangles
// triangleIntersects / triangleIntersect (Primitive/TriangleMesh.hs:140-207)
static inline bool triIntersect(const Prim& pr, const Ray& r, float& t_out, float& b1_out,
                                float& b2_out) {
  V e1 = pr.p2 - pr.p1, e2 = pr.p3 - pr.p1;
  V s1 = cross(r.d, e2);
  float divisor = dot(s1, e1);
  if (divisor == 0) return false;
  float invDiv = 1.0f / divisor;
  V d = r.o - pr.p1;
  float b1 = dot(d, s1) * invDiv;
  if (b1 < 0 || b1 > 1) return false;
  V s2 = cross(d, e1);
  float b2 = dot(r.d, s2) * invDiv;
  if (b2 < 0 || b1 + b2 > 1) return false;
  float t = dot(e2, s2) * invDiv;
  if (t < r.tmin || t > r.tmax) return false;
  t_out = t;
  b1_out = b1;
  b2_out = b2;
  return true;
}

// the rest of triangleIntersect: partial derivatives and the DG (TriangleMesh.hs:182-207)
static void triHitDG(const orc_scene& S, const Prim& pr, const Ray& r, float t, float b1, float b2,
                     DG& dg, float& eps) {
  const Mesh& m = S.meshes[pr.index];
  float uv00 = 0, uv01 = 0, uv10 = 1, uv11 = 0, uv20 = 1, uv21 = 1;  // triangleDefaultUVs
  int o1 = m.idx[3 * pr.tri], o2 = m.idx[3 * pr.tri + 1], o3 = m.idx[3 * pr.tri + 2];
  if (!m.uv.empty()) {
    uv00 = m.uv[2 * o1];
    uv01 = m.uv[2 * o1 + 1];
    uv10 = m.uv[2 * o2];
    uv11 = m.uv[2 * o2 + 1];
    uv20 = m.uv[2 * o3];
    uv21 = m.uv[2 * o3 + 1];
  }
  V e1 = pr.p2 - pr.p1, e2 = pr.p3 - pr.p1;
  V n = normalize(cross(e1, e2));
  float du1 = uv00 - uv20, du2 = uv10 - uv20, dv1 = uv01 - uv21, dv2 = uv11 - uv21;
  V dp1 = pr.p1 - pr.p3, dp2 = pr.p2 - pr.p3;
  float determinant = du1 * dv2 - dv1 * du2;
  V dpdu, dpdv;
  if (determinant == 0) {
    LC c = coordinateSystem(n);
    dpdu = c.s;
    dpdv = c.t;
  } else {
    float invDet = 1.0f / determinant;
    dpdu = sv(invDet, sv(dv2, dp1) - sv(dv1, dp2));
    dpdv = sv(invDet, sv(-du2, dp1) + sv(du1, dp2));
  }
  float b0 = 1.0f - b1 - b2;  // the interpolated (u, v) (TriangleMesh.hs:198-201)
  float tu = b0 * uv00 + b1 * uv10 + b2 * uv20;
  float tv = b0 * uv01 + b1 * uv11 + b2 * uv21;
  dg = mkDg(rayAt(r, t), tu, tv, dpdu, dpdv, V{0, 0, 0}, V{0, 0, 0});
  dg.tri = true;
  dg.b1 = b1;
  dg.b2 = b2;
  eps = 1e-3f * t;
}

// triangleShadingGeometry with o2w = identity (TriangleMesh.hs:122-134);
// Primitive.shadingGeometry is `const` for shapes and normal-less meshes.
static DG shadingGeometry(const orc_scene& S, const Prim& pr, const DG& dgg) {
  if (pr.is_shape) return dgg;
  const Mesh& m = S.meshes[pr.index];
  if (m.n.empty()) return dgg;
  int o1 = m.idx[3 * pr.tri], o2 = m.idx[3 * pr.tri + 1], o3 = m.idx[3 * pr.tri + 2];
  float b1 = dgg.b1, b2 = dgg.b2;
  float b0 = 1.0f - b1 - b2;
  V nsp = sv(b0, m.n[o1]) + sv(b1, m.n[o2]) + sv(b2, m.n[o3]);
  static const float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  V ns = normalize(transNormal(ident, nsp));
  V ssp = normalize(dgg.dpdu);
  V tsp = cross(ssp, ns);
  V ss, ts;
  if (sqLen(tsp) > 0) {
    ss = cross(normalize(tsp), ns);
    ts = normalize(tsp);
  } else {
    LC c = coordinateSystem(ns);
    ss = c.s;
    ts = c.t;
  }
  DG r = dgg;
  r.n = ns;
  r.dpdu = ss;
  r.dpdv = ts;
  return r;
}

struct Hit {
  float t = 0.0f, eps = 0.0f;
  int prim = -1;
  float b1 = 0.0f, b2 = 0.0f;
};

// Primitive.intersect for primitive i, without building the DG (cheap path):
// returns the hit distance only.
static inline bool primHitT(const orc_scene& S, int i, const Ray& r, float& t, float& b1,
                            float& b2) {
  const Prim& pr = S.prims[i];
  if (!pr.is_shape) return triIntersect(pr, r, t, b1, b2);
  const Shape& s = S.shapes[pr.index];
  Ray ro = transRay(s.o2w.i, r);  // mkGeom: transRay w2o (Geometry.hs:33-36)
  float e;
  DG dg;
  b1 = b2 = 0;
  return shapeIntersect(s, ro, t, e, dg);
}
static inline bool primHitAny(const orc_scene& S, int i, const Ray& r) {
  const Prim& pr = S.prims[i];
  if (!pr.is_shape) {
    float t, b1, b2;
    return triIntersect(pr, r, t, b1, b2);
  }
  const Shape& s = S.shapes[pr.index];
  return shapeIntersects(s, transRay(s.o2w.i, r));
}

// closest: the `near` fold over primitives in order (Primitive.hs:29-43)
static bool closestBrute(const orc_scene& S, Ray r, Hit& h) {
  bool any = false;
  for (int i = 0; i < (int)S.prims.size(); i++) {
    float t, b1, b2;
    if (primHitT(S, i, r, t, b1, b2)) {
      r.tmax = t;  // near: rayMax := intDist
      h.t = t;
      h.prim = i;
      h.b1 = b1;
      h.b2 = b2;
      any = true;
    }
  }
  return any;
}
static bool anyBrute(const orc_scene& S, const Ray& r) {
  for (int i = 0; i < (int)S.prims.size(); i++)
    if (primHitAny(S, i, r)) return true;
  return false;
}

// ---- oracle BVH: median split over centroids, boxes widened so traversal
// never prunes a primitive the fold above would hit; ties resolved exactly
// as the fold (smaller t wins, equal t -> larger primitive index).
static AabbF primBounds(const orc_scene& S, int i) {
  const Prim& pr = S.prims[i];
  AabbF b;
  if (!pr.is_shape) {
    b.lo = V{hmin(hmin(pr.p1.x, pr.p2.x), pr.p3.x), hmin(hmin(pr.p1.y, pr.p2.y), pr.p3.y),
             hmin(hmin(pr.p1.z, pr.p2.z), pr.p3.z)};
    b.hi = V{hmax(hmax(pr.p1.x, pr.p2.x), pr.p3.x), hmax(hmax(pr.p1.y, pr.p2.y), pr.p3.y),
             hmax(hmax(pr.p1.z, pr.p2.z), pr.p3.z)};
    return b;
  }
  const Shape& s = S.shapes[pr.index];
  V lo, hi;
  switch (s.kind) {  // objectBounds (Shape.hs:295-311)
    case BLING_SHAPE_BOX: lo = V{s.p[0], s.p[1], s.p[2]}; hi = V{s.p[3], s.p[4], s.p[5]}; break;
    case BLING_SHAPE_CYLINDER: lo = V{-s.p[0], -s.p[0], s.p[1]}; hi = V{s.p[0], s.p[0], s.p[2]}; break;
    case BLING_SHAPE_DISK: lo = V{-s.p[1], -s.p[1], s.p[0]}; hi = V{s.p[1], s.p[1], s.p[0]}; break;
    case BLING_SHAPE_QUAD: lo = V{-s.p[0], -s.p[1], 0}; hi = V{s.p[0], s.p[1], 0}; break;
    default: lo = V{-s.p[0], -s.p[0], -s.p[0]}; hi = V{s.p[0], s.p[0], s.p[0]}; break;
  }
  b.lo = V{INF, INF, INF};
  b.hi = V{-INF, -INF, -INF};
  for (int c = 0; c < 8; c++) {  // transBox (Transform.hs:281-292)
    V q{(c & 4) ? hi.x : lo.x, (c & 2) ? hi.y : lo.y, (c & 1) ? hi.z : lo.z};
    V w = transPoint(s.o2w.m, q);
    b.lo = V{hmin(b.lo.x, w.x), hmin(b.lo.y, w.y), hmin(b.lo.z, w.z)};
    b.hi = V{hmax(b.hi.x, w.x), hmax(b.hi.y, w.y), hmax(b.hi.z, w.z)};
  }
  return b;
}

static void buildOracleBvh(orc_scene& S) {
  int n = (int)S.prims.size();
  S.order.resize(n);
  std::vector<AabbF> bb(n);
  std::vector<V> cen(n);
  for (int i = 0; i < n; i++) {
    S.order[i] = i;
    bb[i] = primBounds(S, i);
    cen[i] = sv(0.5f, bb[i].lo + bb[i].hi);
  }
  S.nodes.clear();
  if (n == 0) return;
  struct Task {
    int node, b, e;
  };
  std::vector<Task> st;
  S.nodes.push_back(BvhNode{});
  st.push_back(Task{0, 0, n});
  while (!st.empty()) {
    Task tk = st.back();
    st.pop_back();
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    double clo[3] = {1e300, 1e300, 1e300}, chi[3] = {-1e300, -1e300, -1e300};
    for (int k = tk.b; k < tk.e; k++) {
      const AabbF& a = bb[S.order[k]];
      const V& c = cen[S.order[k]];
      for (int d = 0; d < 3; d++) {
        lo[d] = std::min(lo[d], (double)comp(a.lo, d));
        hi[d] = std::max(hi[d], (double)comp(a.hi, d));
        clo[d] = std::min(clo[d], (double)comp(c, d));
        chi[d] = std::max(chi[d], (double)comp(c, d));
      }
    }
    BvhNode& nd = S.nodes[tk.node];
    for (int d = 0; d < 3; d++) {
      // widen: hits computed in binary32 may land slightly outside the exact box
      double pad = 1e-4 * (hi[d] - lo[d]) + 1e-5 * std::max(std::fabs(lo[d]), std::fabs(hi[d])) + 1e-30;
      nd.lo[d] = lo[d] - pad;
      nd.hi[d] = hi[d] + pad;
    }
    int cnt = tk.e - tk.b;
    if (cnt <= 4) {
      nd.left = tk.b;
      nd.right = -cnt - 1;
      continue;
    }
    int ax = 0;
    for (int d = 1; d < 3; d++)
      if (chi[d] - clo[d] > chi[ax] - clo[ax]) ax = d;
    int mid = tk.b + cnt / 2;
    std::nth_element(S.order.begin() + tk.b, S.order.begin() + mid, S.order.begin() + tk.e,
                     [&](int a, int b) { return comp(cen[a], ax) < comp(cen[b], ax); });
    int l = (int)S.nodes.size();
    S.nodes.push_back(BvhNode{});
    S.nodes.push_back(BvhNode{});
    S.nodes[tk.node].left = l;
    S.nodes[tk.node].right = l + 1;
    st.push_back(Task{l, tk.b, mid});
    st.push_back(Task{l + 1, mid, tk.e});
  }
}

// slab test in double precision against the widened box
static inline bool nodeHit(const BvhNode& nd, const double o[3], const double inv[3], double t0,
                           double t1) {
  for (int d = 0; d < 3; d++) {
    double a = (nd.lo[d] - o[d]) * inv[d], b = (nd.hi[d] - o[d]) * inv[d];
    if (std::isnan(a) || std::isnan(b)) continue;  // direction 0 and origin on the slab plane
    if (a > b) std::swap(a, b);
    t0 = std::max(t0, a);
    t1 = std::min(t1, b);
  }
  return t0 <= t1;
}

static bool closestBvh(const orc_scene& S, const Ray& r, Hit& h) {
  if (S.nodes.empty()) return false;
  double o[3] = {r.o.x, r.o.y, r.o.z};
  double inv[3] = {1.0 / (double)r.d.x, 1.0 / (double)r.d.y, 1.0 / (double)r.d.z};
  bool any = false;
  float best = r.tmax;
  int bestp = -1;
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  Ray q = r;
  while (sp) {
    const BvhNode& nd = S.nodes[stack[--sp]];
    double tlim = (double)best;
    tlim = tlim + 1e-4 * std::fabs(tlim) + 1e-6;
    if (!nodeHit(nd, o, inv, (double)r.tmin - 1e-6 - 1e-4 * std::fabs((double)r.tmin), tlim)) continue;
    if (nd.right < 0) {
      int cnt = -nd.right - 1;
      for (int k = 0; k < cnt; k++) {
        int pi = S.order[nd.left + k];
        float t, b1, b2;
        q.tmax = best;
        if (primHitT(S, pi, q, t, b1, b2)) {
          if (!any || t < best || (t == best && pi > bestp)) {
            best = t;
            bestp = pi;
            h.t = t;
            h.prim = pi;
            h.b1 = b1;
            h.b2 = b2;
            any = true;
          }
        }
      }
    } else {
      if (sp + 2 > 128) abort();
      stack[sp++] = nd.left;
      stack[sp++] = nd.right;
    }
  }
  return any;
}

static bool anyBvh(const orc_scene& S, const Ray& r) {
  if (S.nodes.empty()) return false;
  double o[3] = {r.o.x, r.o.y, r.o.z};
  double inv[3] = {1.0 / (double)r.d.x, 1.0 / (double)r.d.y, 1.0 / (double)r.d.z};
  double tlo = (double)r.tmin - 1e-6 - 1e-4 * std::fabs((double)r.tmin);
  double thi = (double)r.tmax + 1e-6 + 1e-4 * std::fabs((double)r.tmax);
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const BvhNode& nd = S.nodes[stack[--sp]];
    if (!nodeHit(nd, o, inv, tlo, thi)) continue;
    if (nd.right < 0) {
      int cnt = -nd.right - 1;
      for (int k = 0; k < cnt; k++)
        if (primHitAny(S, S.order[nd.left + k], r)) return true;
    } else {
      if (sp + 2 > 128) abort();
      stack[sp++] = nd.left;
      stack[sp++] = nd.right;
    }
  }
  return false;
}

// ---- the reference's kd-tree (kdtree.h) over the primitives' world bounds
struct KdRay {
  float o[3], d[3], tmin, tmax;
};
static inline KdRay kdRayOf(const Ray& r) {
  return KdRay{{r.o.x, r.o.y, r.o.z}, {r.d.x, r.d.y, r.d.z}, r.tmin, r.tmax};
}

// kdTreePrimitive's intersect (KdTree.hs:240-242): the root interval, then
// traverse with `nearest'` in the leaves
static bool closestKd(const orc_scene& S, const Ray& r0, Hit& h, kd::Counts& c) {
  KdRay r = kdRayOf(r0);
  float tn, tf;
  if (!kd::rootInterval(S.kd.bounds, r.o, r.d, r.tmin, r.tmax, tn, tf)) return false;
  const float inv[3] = {1.0f / r.d[0], 1.0f / r.d[1], 1.0f / r.d[2]};
  bool any = false;
  auto hit = [&](int p, KdRay& kr) {
    Ray q = r0;
    q.tmax = kr.tmax;
    float t, b1, b2;
    if (primHitT(S, p, q, t, b1, b2)) {  // near: rayMax := intDist
      kr.tmax = t;
      h.t = t;
      h.prim = p;
      h.b1 = b1;
      h.b2 = b2;
      any = true;
    }
  };
  kd::closest(S.kd, 0, r, inv, tn, tf, hit, c);
  return any;
}
// kdTreePrimitive's intersects (KdTree.hs:244-246)
static bool anyKd(const orc_scene& S, const Ray& r0, kd::Counts& c) {
  KdRay r = kdRayOf(r0);
  float tn, tf;
  if (!kd::rootInterval(S.kd.bounds, r.o, r.d, r.tmin, r.tmax, tn, tf)) return false;
  const float inv[3] = {1.0f / r.d[0], 1.0f / r.d[1], 1.0f / r.d[2]};
  auto hit = [&](int p, const KdRay&) { return primHitAny(S, p, r0); };
  return kd::any(S.kd, 0, r, inv, tn, tf, hit, c);
}

static void buildKd(orc_scene& S, int nth) {
  std::vector<kd::Box> boxes(S.prims.size());
  for (size_t i = 0; i < S.prims.size(); i++) {
    AabbF b = primBounds(S, (int)i);  // worldBounds of the primitive
    boxes[i] = kd::Box{{b.lo.x, b.lo.y, b.lo.z}, {b.hi.x, b.hi.y, b.hi.z}};
  }
  kd::build(S.kd, boxes, nth);
  S.kd_built = true;
}

struct Isect {
  float t, eps;
  int prim;
  DG dg;  // intGeometry: world-space true geometry
};
// scIntersect returning the full Intersection (Primitive.hs:57-65, Geometry.hs:33-36)
static bool sceneIntersect(const orc_scene& S, const Ray& r, Isect& it) {
  Hit h;
  kd::Counts kc;
  if (!(S.use_kd ? closestKd(S, r, h, kc) : closestBvh(S, r, h))) return false;
  const Prim& pr = S.prims[h.prim];
  it.t = h.t;
  it.prim = h.prim;
  if (!pr.is_shape) {
    triHitDG(S, pr, r, h.t, h.b1, h.b2, it.dg, it.eps);
  } else {
    const Shape& s = S.shapes[pr.index];
    Ray ro = transRay(s.o2w.i, r);
    float t, e;
    DG dg;
    shapeIntersect(s, ro, t, e, dg);
    it.eps = e;
    it.dg = transDg(s.o2w.m, s.o2w.i, dg);
  }
  return true;
}
static bool occluded(const orc_scene& S, const Ray& r) {
  if (S.use_kd) {
    kd::Counts kc;
    return anyKd(S, r, kc);
  }
  return anyBvh(S, r);
}

// ---------------------------------------------------------------- Monte Carlo
// concentricSampleDisk (Montecarlo.hs:160-179)
static void concentricSampleDisk(float u1, float u2, float& ox, float& oy) {
  float sx = u1 * 2.0f - 1.0f, sy = u2 * 2.0f - 1.0f;
  if (sx == 0 && sy == 0) {
    ox = 0;
    oy = 0;
    return;
  }
  float r, thp;
  if (sx >= -sy) {
    if (sx > sy) {
      if (sy > 0) {
        r = sx;
        thp = sy / sx;
      } else {
        r = sx;
        thp = 8.0f + sy / sx;
      }
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
  float theta = thp * PI / 4.0f;
  ox = r * cosf(theta);
  oy = r * sinf(theta);
}
// cosineSampleHemisphere (Montecarlo.hs:146-149)
static V cosineSampleHemisphere(float u1, float u2) {
  float x, y;
  concentricSampleDisk(u1, u2, x, y);
  return V{x, y, sqrtf(hmax(0.0f, 1.0f - x * x - y * y))};
}
// uniformSampleSphere (Montecarlo.hs:181-186)
static V uniformSampleSphere(float u1, float u2) {
  float u = u1 * 2.0f - 1.0f;
  float s = sqrtf(1.0f - (u * u));
  float omega = u2 * 2.0f * PI;
  return V{s * cosf(omega), s * sinf(omega), u};
}
// uniformConePdf / uniformSampleCone (Montecarlo.hs:127-144)
static float uniformConePdf(float cosThetaMax) {
  if (cosThetaMax >= 1) return 0;
  return 1.0f / (TWO_PI * (1.0f - cosThetaMax));
}
static V uniformSampleCone(const LC& c, float cosThetaMax, float u1, float u2) {
  float cosTheta = lerp(u1, cosThetaMax, 1.0f);
  float sinTheta = sqrtf(1.0f - cosTheta * cosTheta);
  float phi = u2 * TWO_PI;
  float a = cosf(phi) * sinTheta, b = sinf(phi) * sinTheta;
  return V{c.s.x * a, c.s.y * a, c.s.z * a} + V{c.t.x * b, c.t.y * b, c.t.z * b} +
         V{c.n.x * cosTheta, c.n.y * cosTheta, c.n.z * cosTheta};
}
// powerHeuristic (Montecarlo.hs:113-116)
static float powerHeuristic(float fPdf, float gPdf) {
  float f = 1.0f * fPdf, g = 1.0f * gPdf;
  return (f * f) / (f * f + g * g);
}
// Dist1D (Montecarlo.hs:34-73)
static void mkDist1D(const std::vector<float>& func, std::vector<float>& cdf, float& fi) {
  int n = (int)func.size();
  std::vector<float> i(n + 1);
  i[0] = 0;
  for (int k = 0; k < n; k++) i[k + 1] = i[k] + func[k] / (float)n;
  fi = i[n];
  cdf.resize(n + 1);
  for (int k = 0; k <= n; k++) cdf[k] = fi != 0 ? i[k] / fi : (float)k / (float)n;
}
static int upperBound(const std::vector<float>& v, float u) {
  int n = (int)v.size();
  int found = -1;
  for (int k = 0; k < n; k++)
    if (v[k] >= u) {
      found = k;
      break;
    }
  int x = found < 0 ? n - 1 : found - 1;
  return std::min(n - 2, std::max(0, x));
}
static void sampleContinuous1D(const std::vector<float>& func, const std::vector<float>& cdf,
                               float fi, float u, float& x, float& pdf, int& off) {
  off = upperBound(cdf, u);
  pdf = fi == 0 ? 0 : func[off] / fi;
  float du = (u - cdf[off]) / (cdf[off + 1] - cdf[off]);
  x = ((float)off + du) / (float)func.size();
}

// ---------------------------------------------------------------- BSDFs
// Reflection.hs:48-88 helpers
static inline float cosTheta(V v) { return v.z; }
static inline float absCosTheta(V v) { return fabsf(v.z); }
static inline float sinTheta2(V v) { return hmax(0.0f, 1.0f - v.z * v.z); }
static inline float sinTheta(V v) { return sqrtf(sinTheta2(v)); }
static inline float cosPhi(V v) {
  float st = sinTheta(v);
  return st == 0 ? 1.0f : clampf(v.x / st, -1, 1);
}
static inline float sinPhi(V v) {
  float st = sinTheta(v);
  return st == 0 ? 0.0f : clampf(v.y / st, -1, 1);
}
static inline bool sameHemisphere(V a, V b) { return a.z * b.z > 0; }
static inline V toSameHemisphere(V wo, V wi) { return wo.z < 0 ? V{wi.x, wi.y, -wi.z} : wi; }

// Fresnel (Fresnel.hs:13-70)
static float frDielScalar(float etai, float etat, float cosi) {
  float c = hmax(0.0f, 1.0f - cosi * cosi);
  float costp = cosi > 0 ? c / (etat * etat) : c * (etat * etat);
  float cost = sqrtf(1.0f - clampf(costp, 0, 1));
  float ac = fabsf(cosi);
  float eta = etat / etai;  // frDiel: etat / etai
  float rParlp = eta * ac;
  float rParl = (cost - rParlp) / (cost + rParlp);
  float rPerpp = eta * cost;
  float rPerp = (ac - rPerpp) / (ac + rPerpp);
  return (rParl * rParl + rPerp * rPerp) * 0.5f;
}
static Spec frEval(const Fresnel& f, float cosi) {
  if (f.kind == FR_NOOP) return WHITE;
  if (f.kind == FR_DIEL) return sConst(frDielScalar(f.ei, f.et, cosi));
  float acosi = fabsf(cosi);
  Spec s;
  for (int i = 0; i < 16; i++) {
    float eta = f.eta.v[i], k = f.k.v[i];
    float tmpF = eta * eta + k * k;
    float tmp = (eta * eta + k * k) * (acosi * acosi);
    float ec2 = eta * (2.0f * acosi);
    float a2 = acosi * acosi;
    float rPer2 = (tmpF - ec2 + a2) / (tmpF + ec2 + a2);
    float rPar2 = (tmp - ec2 + 1.0f) / (tmp + ec2 + 1.0f);
    s.v[i] = (rPer2 + rPar2) / 2.0f;
  }
  return s;
}

// Blinn distribution (Microfacet.hs:113-195)
static float mfG(V wo, V wi, V wh) {
  float nDotWh = absCosTheta(wh), nDotWo = absCosTheta(wo), nDotWi = absCosTheta(wi);
  float woDotWh = absDot(wo, wh);
  return hmin(1.0f, hmin(2.0f * nDotWh * nDotWo / woDotWh, 2.0f * nDotWh * nDotWi / woDotWh));
}
static float blinnPdf(float e, V wh) {
  return (e + 1.0f) * powf(absCosTheta(wh), e) * INV_TWO_PI;
}
static float blinnD(float e, V wh) {
  return (e + 2.0f) * INV_TWO_PI * powf(absCosTheta(wh), e);
}
static void blinnSample(float e, float u1, float u2, V& wh, float& d, float& pdf) {
  float cost = powf(u1, 1.0f / (e + 1.0f));
  float sint = sqrtf(hmax(0.0f, 1.0f - cost * cost));
  float phi = u2 * 2.0f * PI;
  wh = V{sint * cosf(phi), sint * sinf(phi), cost};
  float f = powf(cost, e) * INV_TWO_PI;
  d = (e + 2.0f) * f;
  pdf = (e + 1.0f) * f;
}
static float fixExponent(float e) { return (e > 10000 || std::isnan(e)) ? 10000.0f : e; }

// Oren-Nayar core (Diffuse.hs:53-65)
static Spec orenNayar(const BxDF& b, V wo, V wi) {
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
  return sScale(b.r, b.A + b.B * maxcos * sina * tanb);
}

// bxdfEval b wo wi; a BTDF evaluates its BRDF at the mirrored wi
// the Anisotropic distribution (Microfacet.hs:136-192)
static float anisoPdf(float ex, float ey, V wh) {
  float costh = absCosTheta(wh);
  float e = (ex * wh.x * wh.x + ey * wh.y * wh.y) / hmax(0.0f, 1.0f - costh * costh);
  return sqrtf((ex + 1.0f) * (ey + 1.0f)) * INV_TWO_PI * powf(costh, e);
}
static float anisoD(float ex, float ey, V wh) {
  float costh = absCosTheta(wh);
  float d = 1.0f - costh * costh;
  if (d == 0) return 0;
  float e = (ex * wh.x * wh.x + ey * wh.y * wh.y) / d;
  return sqrtf((ex + 2.0f) * (ey + 2.0f)) * INV_TWO_PI * powf(costh, e);
}
static void anisoSample(float ex, float ey, float u1, float u2, V& wh, float& pdf) {
  auto quad = [&](float up, float& p, float& c) {
    p = ex == ey ? PI * up * 0.5f : atanf(sqrtf((ex + 1.0f) / (ey + 1.0f)) * tanf(PI * up * 0.5f));
    float cp = cosf(p), sp = sinf(p);
    c = powf(u2, 1.0f / (ex * cp * cp + ey * sp * sp + 1.0f));
  };
  float p, cost, phi;
  if (u1 < 0.25f) {
    quad(4.0f * u1, p, cost);
    phi = p;
  } else if (u1 < 0.5f) {
    quad(4.0f * (0.5f - u1), p, cost);
    phi = PI - p;
  } else if (u1 < 0.75f) {
    quad(4.0f * (u1 - 0.5f), p, cost);
    phi = p + PI;
  } else {
    quad(4.0f * (1.0f - u1), p, cost);
    phi = TWO_PI - p;
  }
  float sint = sqrtf(hmax(0.0f, 1.0f - cost * cost));
  wh = V{sint * cosf(phi), sint * sinf(phi), cost};  // sphericalDirection
  float ds = 1.0f - cost * cost;
  float e = (ex * wh.x * wh.x + ey * wh.y * wh.y) / ds;
  float f = INV_TWO_PI * powf(cost, e);
  pdf = sqrtf((ex + 1.0f) * (ey + 1.0f)) * f;
}
// mkFresnelBlend's e wo wi (Microfacet.hs:63-86)
static Spec fblendEval(const BxDF& b, V wo, V wi) {
  float costi = absCosTheta(wi), costo = absCosTheta(wo);
  Spec a = WHITE;
  if (b.e > 0) {
    float x = -(b.e * (costi + costo) / (costi * costo));
    for (int i = 0; i < 16; i++) a.v[i] = expf(b.ra.v[i] * x);
  }
  float ds = ((costo * 28.0f / 23.0f) * PI) * (1.0f - powf(1.0f - 0.5f * costi, 5.0f)) *
             (1.0f - powf(1.0f - 0.5f * costo, 5.0f));
  Spec diff = sScale(a * b.r * (WHITE - b.rs), ds);
  V wh = normalize(wi + wo);
  if (wh.z < 0) wh = -wh;
  float costih = absDot(wi, wh);
  Spec schlick = b.rs + sScale(WHITE - b.rs, powf(1.0f - costih, 5.0f));
  Spec spec = sScale(schlick, anisoD(b.A, b.B, wh) * costo / (4.0f * costih * hmax(costi, costo)));
  return diff + spec;
}

static Spec bxEval(const BxDF& b, V wo, V wi) {
  if (b.btdf) wi = otherHemisphere(wi);
  switch (b.kind) {
    case BX_LAMBERT: return sScale(b.r, INV_PI * absCosTheta(wo));  // Diffuse.hs:26
    case BX_OREN: return sScale(orenNayar(b, wo, wi), INV_PI * absCosTheta(wo));
    case BX_MICRO: {  // Microfacet.hs:21-32
      float costo = absCosTheta(wo), costi = absCosTheta(wi);
      if (costi == 0 || costo == 0) return BLACK;
      V whp = wi + wo;
      if (whp.x == 0 && whp.y == 0 && whp.z == 0) return BLACK;
      V wh = normalize(whp);
      if (cosTheta(wh) < 0) return BLACK;
      float costh = dot(wi, wh);
      float x = blinnD(b.e, wh) * mfG(wo, wi, wh) / (4.0f * costi);
      return sScale(b.r * frEval(b.fr, costh), x);
    }
    case BX_FBLEND: return fblendEval(b, wo, wi);
    default: return BLACK;  // specular: e _ _ = black
  }
}
// bxdfPdf of the BRDF itself
static float bxPdfBrdf(const BxDF& b, V wo, V wi) {
  switch (b.kind) {
    case BX_LAMBERT:
    case BX_OREN: return sameHemisphere(wo, wi) ? INV_PI * absCosTheta(wi) : 0.0f;  // cosPdf
    case BX_MICRO: {
      V whp = wo + wi;
      if (sqLen(whp) == 0) return 0;
      V wh = normalize(whp);
      if (cosTheta(wh) < 0) return 0;
      return blinnPdf(b.e, wh) / (4.0f * absDot(wo, wh));
    }
    case BX_FBLEND: {  // Microfacet.hs:104-108
      if (!sameHemisphere(wo, wi)) return 0;
      V wh = normalize(wi + wo);
      if (wh.z < 0) wh = -wh;
      return 0.5f * (absCosTheta(wi) * INV_PI + anisoPdf(b.A, b.B, wh) / (4.0f * absDot(wo, wh)));
    }
    default: return 0;
  }
}
// bxdfPdf b wo wi
static float bxPdf(const BxDF& b, V wo, V wi) {
  return bxPdfBrdf(b, wo, b.btdf ? otherHemisphere(wi) : wi);
}
static void bxSampleBrdf(const BxDF& b, V wo, float u1, float u2, Spec& f, V& wi, float& pdf,
                         bool adj);
// bxdfSample b adj wo u -> (f, wi, pdf); a BTDF mirrors its BRDF's sample
// (Reflection.hs:188-195).  adj: the adjoint (light-to-camera) transport
static void bxSample(const BxDF& b, V wo, float u1, float u2, Spec& f, V& wi, float& pdf,
                     bool adj = false) {
  bxSampleBrdf(b, wo, u1, u2, f, wi, pdf, adj);
  if (b.btdf) wi = otherHemisphere(wi);
}
static void bxSampleBrdf(const BxDF& b, V wo, float u1, float u2, Spec& f, V& wi, float& pdf,
                         bool adj) {
  switch (b.kind) {
    case BX_LAMBERT: {  // cosSample (Diffuse.hs:14-22)
      wi = toSameHemisphere(wo, cosineSampleHemisphere(u1, u2));
      if (sameHemisphere(wo, wi)) {
        f = adj ? sScale(b.r, fabsf(cosTheta(wo) / cosTheta(wi))) : b.r;
        pdf = bxPdfBrdf(b, wo, wi);
      } else {
        f = BLACK;
        wi = wo;
        pdf = 0;
      }
      return;
    }
    case BX_OREN: {  // Diffuse.hs:38-49
      wi = toSameHemisphere(wo, cosineSampleHemisphere(u1, u2));
      if (sameHemisphere(wo, wi)) {
        f = adj ? sScale(orenNayar(b, wo, wi), fabsf(cosTheta(wo) / cosTheta(wi)))
                : orenNayar(b, wo, wi);
        pdf = bxPdfBrdf(b, wo, wi);
      } else {
        f = BLACK;
        pdf = 0;
      }
      return;
    }
    case BX_FBLEND: {  // Microfacet.hs:88-102
      V wh;
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
        f = BLACK;
        pdf = 0;
        return;
      }
      pdf = 0.5f * (absCosTheta(wi) * INV_PI + pdfp / (4.0f * absDot(wo, wh)));
      f = sScale(adj ? fblendEval(b, wi, wo) : fblendEval(b, wo, wi), 1.0f / pdf);
      return;
    }
    case BX_SPEC_REFL: {  // Specular.hs:11-20
      f = b.r * frEval(b.fr, cosTheta(wo));
      wi = V{-wo.x, -wo.y, wo.z};
      pdf = 1;
      return;
    }
    case BX_SPEC_TRANS: {  // sampleSpecTrans (Specular.hs:35-58)
      bool entering = cosTheta(wo) > 0;
      float ei = entering ? b.ei : b.et, et = entering ? b.et : b.ei;
      float sini2 = sinTheta2(wo);
      float eta = ei / et;
      float eta2 = eta * eta;
      float sint2 = eta2 * sini2;
      if (sint2 >= 1) {
        f = BLACK;
        wi = wo;
        pdf = 0;
        return;
      }
      float c = sqrtf(hmax(0.0f, 1.0f - sint2));
      float cost = entering ? -c : c;
      wi = V{eta * (-wo.x), eta * (-wo.y), cost};
      Spec fr = sConst(frDielScalar(ei, et, adj ? cosTheta(wo) : cost));
      f = adj ? sScale((WHITE - fr) * b.r, fabsf(cosTheta(wo) / cost)) : sScale((WHITE - fr) * b.r, eta2);
      pdf = 1;
      return;
    }
    default: {  // microfacet (Microfacet.hs:42-54)
      V whp;
      float d, p;
      blinnSample(b.e, u1, u2, whp, d, p);
      V wh = cosTheta(whp) < 0 ? -whp : whp;
      wi = sv(2.0f * dot(wo, wh), wh) - wo;
      float costH = dot(wo, wh);
      float fact = d * fabsf(costH) / p * mfG(wo, wi, wh);
      Spec fp = b.r * frEval(b.fr, costH);
      if (sameHemisphere(wo, wi)) {
        f = sScale(fp, fact / absCosTheta(adj ? wo : wi));
        pdf = p / (4.0f * fabsf(costH));
      } else {
        f = BLACK;
        wi = wo;
        pdf = 0;
      }
      return;
    }
  }
}

struct Bsdf {  // Reflection.hs:201-218
  BxDF c[2];
  int n;
  LC cs;
  V p;
  V ng;
};

// mkBsdf' with the material's BxDFs (Material.hs:32-127)
// frApproxEta / frApproxK (Fresnel.hs:72-78), on sClamp 0 0.999 of the colour
static Spec frApproxEta(const Spec& r) {
  Spec c = sClamp(0.0f, 0.999f, r), o;
  for (int i = 0; i < 16; i++) {
    float rs = std::sqrt(c.v[i]);
    o.v[i] = (1.0f + rs) / (1.0f - rs);
  }
  return o;
}
static Spec frApproxK(const Spec& r) {
  Spec c = sClamp(0.0f, 0.999f, r), o;
  for (int i = 0; i < 16; i++) o.v[i] = std::sqrt(c.v[i] / (1.0f - c.v[i])) * 2.0f;
  return o;
}

// ---------------------------------------------------------------- textures
// Texture.hs restated: the mappings, Perlin noise and fBm, Worley cell noise,
// the quasi-crystal, gradients, blends, checkers, graph paper and images.
static const uint8_t NOISE_PERM[256] = {BLING_NOISE_PERM_LIST};

// noiseWeight (Texture.hs:378-382)
static float noiseWeight(float t) {
  float t3 = t * t * t;
  float t4 = t3 * t;
  return 6.0f * t4 * t - 15.0f * t4 + 10.0f * t3;
}
// grad (Texture.hs:384-393); noisePerms is the permutation written twice
static float grad(int x, int y, int z, float dx, float dy, float dz) {
  auto P = [](int i) { return (int)NOISE_PERM[i % 256]; };
  int h = P(P(P(x) + y) + z) & 15;
  float u = (h < 8 || h == 12 || h == 13) ? dx : dy;
  float v = (h < 4 || h == 12 || h == 13) ? dy : dz;
  return ((h & 1) != 0 ? -u : u) + ((h & 2) != 0 ? -v : v);
}
// perlin3d (Texture.hs:348-376)
static float perlin3d(float x, float y, float z) {
  long long ix0 = (long long)std::floor(x), iy0 = (long long)std::floor(y),
            iz0 = (long long)std::floor(z);
  float dx = x - (float)ix0, dy = y - (float)iy0, dz = z - (float)iz0;
  int ix = (int)(ix0 & 255), iy = (int)(iy0 & 255), iz = (int)(iz0 & 255);
  float w000 = grad(ix, iy, iz, dx, dy, dz);
  float w100 = grad(ix + 1, iy, iz, dx - 1, dy, dz);
  float w010 = grad(ix, iy + 1, iz, dx, dy - 1, dz);
  float w110 = grad(ix + 1, iy + 1, iz, dx - 1, dy - 1, dz);
  float w001 = grad(ix, iy, iz + 1, dx, dy, dz - 1);
  float w101 = grad(ix + 1, iy, iz + 1, dx - 1, dy, dz - 1);
  float w011 = grad(ix, iy + 1, iz + 1, dx, dy - 1, dz - 1);
  float w111 = grad(ix + 1, iy + 1, iz + 1, dx - 1, dy - 1, dz - 1);
  float wx = noiseWeight(dx), wy = noiseWeight(dy), wz = noiseWeight(dz);
  float x00 = lerp(wx, w000, w100), x10 = lerp(wx, w010, w110);
  float x01 = lerp(wx, w001, w101), x11 = lerp(wx, w011, w111);
  return lerp(wz, lerp(wy, x00, x10), lerp(wy, x01, x11));
}
// fbm (Texture.hs:328-337): sum (take octaves terms), the sum a left fold from 0
static float fbm(int octaves, float omega, V p) {
  float sum = 0.0f, l = 1.0f, o = 1.0f;
  for (int k = 0; k < octaves; k++) {
    sum = sum + o * perlin3d(p.x * l, p.y * l, p.z * l);
    l = 1.99f * l;  // iterate (1.99 *) 1
    o = omega * o;  // iterate (omega *) 1
  }
  return sum;
}
// cellNoise (Texture.hs:250-300): Int is 64 bits
static float cellNoise(int dist, V p) {
  auto lcg = [](long long x) { return (1103515245LL * x + 12345LL) % 4294967296LL; };
  auto hash = [](long long x, long long y, long long z) {
    long long h = (x * 73856093LL) ^ (y * 19349663LL) ^ (z * 83492791LL);
    return std::llabs(h) % 4294967296LL;
  };
  auto prob = [](long long v) {
    static const long long lim[8] = {393325350LL,  1022645910LL, 1861739990LL, 2700834071LL,
                                     3372109335LL, 3819626178LL, 4075350088LL, 4203212043LL};
    for (int k = 0; k < 8; k++)
      if (v < lim[k]) return k + 1;
    return 9;
  };
  auto distf = [&](V a, V b) {
    V d = a - b;
    switch (dist) {
      case BLING_DIST_EUCLIDIAN2: return sqLen(d);
      case BLING_DIST_MANHATTAN: return fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
      case BLING_DIST_CHEBYSHEV: return hmax(hmax(fabsf(d.x), fabsf(d.y)), fabsf(d.z));
      default: return len(d);
    }
  };
  long long ox = (long long)std::floor(p.x), oy = (long long)std::floor(p.y),
            oz = (long long)std::floor(p.z);
  std::vector<float> ds;
  for (int x = -1; x <= 1; x++)
    for (int y = -1; y <= 1; y++)
      for (int z = -1; z <= 1; z++) {
        long long cx = x + ox, cy = y + oy, cz = z + oz;
        long long us = lcg(hash(cx, cy, cz));
        int n = prob(us);
        long long u0 = us;
        for (int k = 0; k < n; k++) {
          long long u1 = lcg(u0), u2 = lcg(u1), u3 = lcg(u2);
          V pt{(float)cx + (float)u1 / 4294967296.0f, (float)cy + (float)u2 / 4294967296.0f,
               (float)cz + (float)u3 / 4294967296.0f};
          ds.push_back(distf(p, pt));
          u0 = u3;
        }
      }
  float m = ds[0];  // minimum = foldl1 min
  for (size_t k = 1; k < ds.size(); k++) m = hmin(m, ds[k]);
  return m;
}
// quasiCrystal (Texture.hs:302-326); the angles as base-4.9's
// numericEnumFromThen makes them (each next one m + m - n)
static float quasiCrystal(int octaves, float x, float y) {
  std::vector<float> angles;
  float n0 = 0.0f, m0 = PI / (float)octaves;
  for (int k = 0; k < octaves; k++) {
    angles.push_back(n0);
    float nx = m0 + m0 - n0;
    n0 = m0;
    m0 = nx;
  }
  float sum = 0.0f;
  for (float th : angles) {
    float cth = cosf(th), sth = sinf(th);
    sum = sum + (cosf(cth * x + sth * y) + 1.0f) / 2.0f;
  }
  long long k = (long long)sum;  // properFraction: truncation
  float v = sum - (float)k;
  if (v < 0) {
    k = k - 1;
    v = 1.0f + v;
  }
  return (k % 2 != 0) ? 1.0f - v : v;
}

struct TexPoint {  // what textures read of the shading DG
  V p;
  float u, v;
};
// uvMapping / planarMapping (Texture.hs:160-176)
static void map2d(const TexNode& t, const TexPoint& g, float& s, float& r) {
  if (t.map_kind == BLING_MAP_PLANAR) {
    s = dot(g.p, V{t.map[0], t.map[1], t.map[2]}) + t.map[6];
    r = dot(g.p, V{t.map[3], t.map[4], t.map[5]}) + t.map[7];
  } else {
    s = t.map[0] * g.u + t.map[2];
    r = t.map[1] * g.v + t.map[3];
  }
}
// identityMapping3d (Texture.hs:150-154)
static V map3d(const TexNode& t, const TexPoint& g) { return transPoint(t.map, g.p); }
// getPixel's pixel index (Texture.hs:91-101): mod' (floor (u w)) w,
// mod' (floor (-v h)) h
static size_t pixelIndex(const TexNode& t, float s, float r) {
  auto modp = [](long long a, long long b) {
    long long q = a / b, rem = a - q * b;
    if (rem != 0 && ((rem < 0) != (b < 0))) rem += b;  // Haskell's div floors
    return rem;
  };
  long long px = modp((long long)std::floor(s * (float)t.w), t.w);
  long long py = modp((long long)std::floor((-r) * (float)t.h), t.h);
  return (size_t)py * t.w + (size_t)px;
}

static float scalarTex(const orc_scene& S, int i, const TexPoint& g) {
  const TexNode& t = S.tex[i];
  switch (t.kind) {
    case BLING_TEXN_SCALE: return t.p[0] + t.p[1] * scalarTex(S, t.a, g);
    case BLING_TEXN_PERLIN: {
      V q = map3d(t, g);
      return perlin3d(q.x, q.y, q.z);
    }
    case BLING_TEXN_FBM: return fbm(t.ivalue, t.p[0], map3d(t, g));
    case BLING_TEXN_CELL_NOISE: return cellNoise(t.ivalue, map3d(t, g));
    case BLING_TEXN_CRYSTAL: {
      float s, r;
      map2d(t, g, s, r);
      return quasiCrystal(t.ivalue, s, r);
    }
    case BLING_TEXN_IMAGE_SCALAR: {  // getPixelScalar: x / 255
      float s, r;
      map2d(t, g, s, r);
      return (float)t.pixels[pixelIndex(t, s, r)] / 255.0f;
    }
    default: return t.p[0];
  }
}
static Spec spectrumTex(const orc_scene& S, int i, const TexPoint& g) {
  const TexNode& t = S.tex[i];
  switch (t.kind) {
    case BLING_TEXN_BLEND: {  // spectrumBlend
      Spec v1 = spectrumTex(S, t.a, g), v2 = spectrumTex(S, t.b, g);
      float x = scalarTex(S, t.c, g);
      if (x <= 0) return v1;
      if (x >= 1) return v2;
      return sScale(v1, 1.0f - x) + sScale(v2, x);
    }
    case BLING_TEXN_CHECKER: {  // checkerBoard: Haskell's mod 2 of the floor sum
      long long c = (long long)std::floor(g.p.x * t.p[0]) + (long long)std::floor(g.p.y * t.p[1]) +
                    (long long)std::floor(g.p.z * t.p[2]);
      return ((c % 2) + 2) % 2 == 0 ? spectrumTex(S, t.a, g) : spectrumTex(S, t.b, g);
    }
    case BLING_TEXN_GRAPH_PAPER: {
      float x, z;
      map2d(t, g, x, z);
      float xf = fabsf(x - (float)(long long)x), zf = fabsf(z - (float)(long long)z);
      float lo = t.p[0] / 2.0f, hi = 1.0f - lo;
      return (xf < lo || zf < lo || xf > hi || zf > hi) ? spectrumTex(S, t.b, g)
                                                        : spectrumTex(S, t.a, g);
    }
    case BLING_TEXN_GRADIENT: {
      float f = scalarTex(S, t.c, g);
      int n = t.ivalue;
      auto pos = [&](int k) { return t.steps[17 * k]; };
      auto col = [&](int k) {
        Spec c;
        memcpy(c.v, &t.steps[17 * k + 1], 64);
        return c;
      };
      float gmin = pos(0), gmax = pos(0);  // V.minimum / V.maximum of the positions
      for (int k = 1; k < n; k++) {
        gmin = hmin(gmin, pos(k));
        gmax = hmax(gmax, pos(k));
      }
      if (f <= gmin) return col(0);
      if (f >= gmax) return col(n - 1);
      int idx = 0;
      while (idx < n && !(pos(idx) > f)) idx++;  // findIndex ((> f) . fst)
      float w = (f - pos(idx - 1)) / (pos(idx) - pos(idx - 1));
      return sScale(col(idx - 1), 1.0f - w) + sScale(col(idx), w);
    }
    case BLING_TEXN_IMAGE: {  // pixelSpectrum = rgbToSpectrumRefl . unGamma
      float s, r;
      map2d(t, g, s, r);
      const uint8_t* px = &t.pixels[3 * pixelIndex(t, s, r)];
      float c[3];
      for (int k = 0; k < 3; k++) c[k] = powf((float)px[k] / 255.0f, 2.2f);
      return rgbToSpectrum(false, c[0], c[1], c[2]);
    }
    default: return t.spectrum;
  }
}

// bump (Reflection.hs:347-377) of dgs by the scalar node d; dgg's normal
// orients the result
static void bump(const orc_scene& S, int d, const DG& dgg, DG& dgs) {
  const float du = 0.01f, dv = 0.01f;
  TexPoint geu{dgs.p + sv(du, dgs.dpdu), dgs.u + du, dgs.v};
  TexPoint gev{dgs.p + sv(dv, dgs.dpdv), dgs.u, dgs.v + dv};
  TexPoint gs{dgs.p, dgs.u, dgs.v};
  float uDisp = scalarTex(S, d, geu), vDisp = scalarTex(S, d, gev), disp = scalarTex(S, d, gs);
  float vscale = (vDisp - disp) / dv;
  V dpdv = dgs.dpdv + sv(vscale, dgs.n);
  float uscale = (uDisp - disp) / du;
  V dpdu = dgs.dpdu + sv(uscale, dgs.n);
  V nn = normalize(cross(dpdu, dpdv));
  if (dot(nn, dgg.n) < 0) nn = -nn;  // faceForward
  dgs.n = nn;
  dgs.dpdu = dpdu;
  dgs.dpdv = dpdv;
}

// the material at a hit: bumpMapped applies its bump to dgs, then every
// textured parameter is its texture at dgs
static Material hitMaterial(const orc_scene& S, int mi, const DG& dgg, DG& dgs) {
  Material m = S.mats[mi];
  if (m.bump) bump(S, m.bump - 1, dgg, dgs);
  TexPoint g{dgs.p, dgs.u, dgs.v};
  Spec* spectra[5] = {&m.kd, &m.ks, &m.kt, &m.eta, &m.k};
  for (int k = 0; k < 5; k++)
    if (m.tex[k]) *spectra[k] = spectrumTex(S, m.tex[k] - 1, g);
  if (m.tex[0]) m.kd_tex = BLING_TEX_CONSTANT;
  if (m.tex[5]) m.sigma = scalarTex(S, m.tex[5] - 1, g);
  if (m.tex[6]) m.rough = scalarTex(S, m.tex[6] - 1, g);
  if (m.tex[7]) m.ior = scalarTex(S, m.tex[7] - 1, g);
  return m;
}

static Bsdf materialBsdf(const Material& m0, const DG& dgg, const DG& dgs) {
  // the kd texture at the shading point
  const Material& m = m0;
  const Spec* kdp = &m.kd;  // the textured diffuse colour of matte, plastic, substrate
  if (m.kd_tex == BLING_TEX_CHECKER) {  // checkerBoard (Texture.hs:209-219)
    long long c = (long long)floorf(dgs.p.x * m.kd_par[0]) + (long long)floorf(dgs.p.y * m.kd_par[1]) +
                  (long long)floorf(dgs.p.z * m.kd_par[2]);
    if (((c % 2) + 2) % 2 == 1) kdp = &m.kd2;
  } else if (m.kd_tex == BLING_TEX_GRAPH_PAPER) {  // graphPaper + planarMapping (Texture.hs:172-207)
    const float* q = m.kd_par;
    float u = dot(dgs.p, V{q[1], q[2], q[3]}) + q[7], v = dot(dgs.p, V{q[4], q[5], q[6]}) + q[8];
    float xf = fabsf(u - truncf(u)), zf = fabsf(v - truncf(v));  // properFraction
    float lo = q[0] / 2.0f, hi = 1.0f - lo;
    if (xf < lo || zf < lo || xf > hi || zf > hi) kdp = &m.kd2;
  }
  Bsdf b;
  b.n = 0;
  V nn = dgs.n, sn = normalize(dgs.dpdu);
  b.cs = LC{sn, cross(nn, sn), nn};
  b.p = dgs.p;
  b.ng = dgg.n;
  auto add = [&](const BxDF& x) { b.c[b.n++] = x; };
  BxDF x{};
  switch (m.kind) {
    case BLING_MAT_MATTE:
      if (m.sigma == 0) {
        x.kind = BX_LAMBERT;
        x.type = T_REFL | T_DIFF;
        x.r = *kdp;
      } else {
        x.kind = BX_OREN;
        x.type = T_REFL | T_DIFF;
        x.r = *kdp;
        float s = clampf(m.sigma, 0, 1);
        float sig2 = s * s;
        x.A = 1.0f - (sig2 / (2.0f * (sig2 + 0.33f)));
        x.B = 0.45f * sig2 / (sig2 + 0.09f);
      }
      add(x);
      break;
    case BLING_MAT_PLASTIC: {
      x.kind = BX_LAMBERT;
      x.type = T_REFL | T_DIFF;
      x.r = *kdp;
      add(x);
      BxDF y{};
      y.kind = BX_MICRO;
      y.type = T_REFL | T_GLOSSY;
      y.r = m.ks;
      y.e = fixExponent(1.0f / m.rough);
      y.fr.kind = FR_DIEL;
      y.fr.ei = 1.0f;
      y.fr.et = 1.5f;
      add(y);
      break;
    }
    case BLING_MAT_METAL: {
      x.kind = BX_MICRO;
      x.type = T_REFL | T_GLOSSY;
      x.r = WHITE;
      x.e = fixExponent(1.0f / m.rough);
      x.fr.kind = FR_COND;
      x.fr.eta = m.eta;
      x.fr.k = m.k;
      add(x);
      break;
    }
    case BLING_MAT_SHINY_METAL: {  // mkShinyMetal kr ks rough (Material.hs:98-109)
      x.kind = BX_MICRO;
      x.type = T_REFL | T_GLOSSY;
      x.r = WHITE;
      x.e = fixExponent(1.0f / m.rough);
      x.fr.kind = FR_COND;
      x.fr.eta = frApproxEta(m.ks);
      x.fr.k = frApproxK(m.ks);
      add(x);
      BxDF y{};
      y.kind = BX_SPEC_REFL;
      y.type = T_REFL | T_SPEC;
      y.r = WHITE;
      y.fr.kind = FR_COND;
      y.fr.eta = frApproxEta(m.kd);  // kr
      y.fr.k = frApproxK(m.kd);
      add(y);
      break;
    }
    case BLING_MAT_BLACKBODY:  // blackBodyMaterial (Reflection.hs:337-338): no BxDFs
      break;
    case BLING_MAT_SUBSTRATE: {  // mkSubstrate kd ks ka u v depth (Material.hs:111-127)
      x.kind = BX_FBLEND;
      x.type = T_REFL | T_GLOSSY;
      x.r = sClamp(0, 1, *kdp);
      x.rs = sClamp(0, 1, m.ks);
      x.ra = sClamp(0, 1, m.kt);  // ka
      float u = hmax(0.0f, m.rough), v = hmax(0.0f, m.sigma);
      x.A = fixExponent(1.0f / u);  // mkAnisotropic (1 / u) (1 / v)
      x.B = fixExponent(1.0f / v);
      x.e = m.ior;  // coating depth
      add(x);
      break;
    }
    case BLING_MAT_TRANS_MATTE: {  // translucentMatte kr kt ks (Material.hs:43-53)
      Spec r = sClamp(0, 1, m.kd);
      Spec t = sClamp(0, 1, m.kt) * (WHITE - r);
      x.type = T_REFL | T_DIFF;
      x.r = r;
      if (m.sigma == 0) {
        x.kind = BX_LAMBERT;
      } else {
        x.kind = BX_OREN;
        float sg = clampf(m.sigma, 0, 1);
        float sig2 = sg * sg;
        x.A = 1.0f - (sig2 / (2.0f * (sig2 + 0.33f)));
        x.B = 0.45f * sig2 / (sig2 + 0.09f);
      }
      add(x);
      BxDF y = x;
      y.type = T_TRANS | T_DIFF;
      y.r = t;
      y.btdf = true;
      add(y);
      break;
    }
    case BLING_MAT_MIRROR: {  // mirrorMaterial: specRefl frNoOp (sClamp 0 1 kr)
      x.kind = BX_SPEC_REFL;
      x.type = T_REFL | T_SPEC;
      x.r = sClamp(0, 1, m.ks);
      x.fr.kind = FR_NOOP;
      add(x);
      break;
    }
    default: {  // glass
      x.kind = BX_SPEC_REFL;
      x.type = T_REFL | T_SPEC;
      x.r = sClamp(0, 1, m.ks);
      x.fr.kind = FR_DIEL;
      x.fr.ei = 1.0f;
      x.fr.et = m.ior;
      add(x);
      BxDF y{};
      y.kind = BX_SPEC_TRANS;
      y.type = T_TRANS | T_SPEC;
      y.r = sClamp(0, 1, m.kt);
      y.ei = 1.0f;
      y.et = m.ior;
      add(y);
      break;
    }
  }
  return b;
}

struct BsdfSample {
  int type;
  float pdf;
  Spec f;
  V wi;
};

// sampleBsdf'' adj bxdfAll (Reflection.hs:278-316); adj = True is
// sampleAdjBsdf (Reflection.hs:272-273)
static BsdfSample sampleBsdf(const Bsdf& b, V woW, float uComp, float u1, float u2,
                             bool adj = false) {
  BsdfSample empty{T_REFL | T_DIFF, 0, BLACK, V{0, 1, 0}};
  if (b.n == 0) return empty;
  V wo = worldToLocal(b.cs, woW);
  int cntm = b.n;
  float cntf = (float)cntm;
  float invCnt = 1.0f / cntf;
  int sNum = std::max(0, std::min(cntm - 1, (int)floorf(uComp * cntf)));
  const BxDF& bx = b.c[sNum];
  Spec fSample;
  V wi;
  float pdfp;
  bxSample(bx, wo, u1, u2, fSample, wi, pdfp, adj);
  V wiW = localToWorld(b.cs, wi);
  float sideTest = dot(wiW, b.ng) / dot(woW, b.ng);
  if (pdfp == 0 || sideTest == 0) return empty;
  bool wantTrans = sideTest < 0;
  auto flt = [&](const BxDF& x) { return wantTrans ? (x.type & T_TRANS) != 0 : (x.type & T_REFL) != 0; };
  if (!flt(bx)) return empty;
  // fAdj: the adjoint's correction for shading normals
  auto fAdj = [&](const Spec& ff) { return adj ? sScale(ff, fabsf(sideTest)) : ff; };
  if (bx.type & T_SPEC) return BsdfSample{bx.type, pdfp * invCnt, sScale(fAdj(fSample), cntf), wiW};
  if (cntm == 1) return BsdfSample{bx.type, pdfp, fAdj(fSample), wiW};
  float others = 0.0f;
  for (int i = 0; i < cntm; i++)
    if (i != sNum) others = others + bxPdf(b.c[i], wo, wi);
  float pdf = (pdfp + others) * invCnt;
  Spec fOthers = BLACK;
  for (int i = 0; i < cntm; i++)
    if (i != sNum && flt(b.c[i]))
      fOthers = fOthers + (adj ? bxEval(b.c[i], wo, wi) : bxEval(b.c[i], wi, wo));  // flip unless adj
  Spec fSum = sScale(sScale(fSample, pdfp) + fOthers, 1.0f / pdf);
  return BsdfSample{bx.type, pdf, fAdj(fSum), wiW};
}
// evalBsdf adj (Reflection.hs:318-332)
static Spec evalBsdf(const Bsdf& b, V woW, V wiW, bool adj = false) {
  float cosWo = dot(woW, b.ng);
  float sideTest = dot(wiW, b.ng) / cosWo;
  if (sideTest == 0) return BLACK;
  if (fabsf(cosWo) < 1e-5f) return BLACK;
  bool wantTrans = sideTest < 0;
  V wo = worldToLocal(b.cs, woW), wi = worldToLocal(b.cs, wiW);
  Spec f = BLACK;
  for (int i = 0; i < b.n; i++) {
    const BxDF& x = b.c[i];
    bool ok = wantTrans ? (x.type & T_TRANS) != 0 : (x.type & T_REFL) != 0;
    if (ok) f = f + (adj ? bxEval(x, wo, wi) : bxEval(x, wi, wo));  // flip (bxdfEval b) unless adj
  }
  return adj ? sScale(f, fabsf(sideTest)) : f;  // shading-normal correction of the adjoint
}
// bsdfPdf (Reflection.hs:251-257)
static float bsdfPdf(const Bsdf& b, V woW, V wiW) {
  if (b.n == 0) return 0;
  V wo = worldToLocal(b.cs, woW), wi = worldToLocal(b.cs, wiW);
  float s = 0.0f;
  for (int i = 0; i < b.n; i++) s = s + bxPdf(b.c[i], wo, wi);
  return s / (float)b.n;
}

// ---------------------------------------------------------------- lights
// sampleShape' / sampleShape (Shape.hs:362-409), local space
static bool insideSphere(float r, V p) { return sqLen(p) - r * r < 1e-4f; }
static void sampleShapeP(const Shape& s, float u1, float u2, V& p, V& n) {
  switch (s.kind) {
    case BLING_SHAPE_BOX: {
      int axis = std::min(2, (int)floorf(u1 * 3.0f));
      float u1p = (u1 - (float)axis / 3.0f) * 3.0f;  // remapRand 3 (Math.hs:113-121)
      int nf = std::min(1, (int)floorf(u2 * 2.0f));
      float u2p = (u2 - (float)nf / 2.0f) * 2.0f;
      n = setComp(axis, (float)nf * 2.0f - 1.0f, mkV(0, 0, 0));
      int oa0 = (axis + 1) % 3, oa1 = (axis + 2) % 3;
      V pmin{s.p[0], s.p[1], s.p[2]}, pmax{s.p[3], s.p[4], s.p[5]};
      V base = nf == 0 ? pmin : pmax;
      p = setComp(oa0, lerp(u1p, comp(pmin, oa0), comp(pmax, oa0)),
                  setComp(oa1, lerp(u2p, comp(pmin, oa1), comp(pmax, oa1)), base));
      return;
    }
    case BLING_SHAPE_CYLINDER: {
      float z = lerp(u1, s.p[1], s.p[2]);
      float phi = lerp(u2, 0, TWO_PI);
      p = V{s.p[0] * cosf(phi), s.p[0] * sinf(phi), z};
      n = normalize(V{p.x, p.y, 0});
      return;
    }
    case BLING_SHAPE_DISK: {
      float r = lerp(u1, s.p[2], s.p[1]);
      float phi = lerp(u2, 0, s.p[3]);
      p = V{r * cosf(phi), r * sinf(phi), s.p[0]};
      n = V{0, 0, -1};
      return;
    }
    case BLING_SHAPE_QUAD:
      p = V{lerp(u1, -s.p[0], s.p[0]), lerp(u2, -s.p[1], s.p[1]), 0};
      n = V{0, 0, -1};
      return;
    default: {
      V q = uniformSampleSphere(u1, u2);
      p = q * V{s.p[0], s.p[0], s.p[0]};
      n = q;
      return;
    }
  }
}
static void sampleShape(const Shape& s, V pt, float u1, float u2, V& ps, V& ns) {
  if (s.kind == BLING_SHAPE_SPHERE && !insideSphere(s.p[0], pt)) {
    float r = s.p[0];
    V dn = normalize(-pt);
    LC cs = coordinateSystem(dn);
    float cosThetaMax = sqrtf(hmax(0.0f, 1.0f - (r * r) / sqLen(pt)));
    V d = uniformSampleCone(cs, cosThetaMax, u1, u2);
    Ray ray{pt, d, 0, INF};
    float t, e;
    DG dg;
    ps = shapeIntersect(s, ray, t, e, dg) ? rayAt(ray, t) : dn * V{r, r, r};
    ns = normalize(ps);
    return;
  }
  sampleShapeP(s, u1, u2, ps, ns);
}
// shapePdf / generalPdf (Shape.hs:333-350)
static float generalPdf(const Shape& s, V p, V wi) {
  Ray r{p, wi, 1e-3f, INF};
  float t, e;
  DG dg;
  if (!shapeIntersect(s, r, t, e, dg)) return 0;
  float pd = sqLen(p - rayAt(r, t)) / (absDot(dg.n, -wi) * shapeArea(s));
  return std::isinf(pd) ? 0.0f : pd;
}
static float shapePdf(const Shape& s, V p, V wi) {
  if (s.kind == BLING_SHAPE_SPHERE && !insideSphere(s.p[0], p)) {
    float r = s.p[0];
    float sinThetaMax2 = r * r / sqLen(p);
    float cosThetaMax = sqrtf(hmax(0.0f, 1.0f - sinThetaMax2));
    return uniformConePdf(cosThetaMax);
  }
  return generalPdf(s, p, wi);
}

// spherical helpers (Math.hs:141-169, Types.hs:31-39)
static V sphericalDirection(float sint, float cost, float phi) {
  return V{sint * cosf(phi), sint * sinf(phi), cost};
}
static float sphericalTheta(V v) { return acosf(hmax(-1.0f, hmin(1.0f, v.z))); }
static float sphericalPhi(V v) {
  float p = hatan2(v.y, v.x);
  return p < 0 ? p + 2.0f * PI : p;
}
// the lat-long map lookup: nearest texel (u in [0,1) across, v in [0,1) down)
// of an image map, or the sun/sky function at (u, v)
static Spec envLookup(const Light& l, float u, float v) {
  if (l.sky) return sunSkyEval(l.skyd, u, v);
  int x = (int)floorf(u * (float)l.w), y = (int)floorf(v * (float)l.h);
  x = std::max(0, std::min(l.w - 1, x));
  y = std::max(0, std::min(l.h - 1, y));
  return l.env[(size_t)y * l.w + x];
}

struct LightSample {  // Light.hs:23-29
  Spec li;
  V wi;
  Ray ray;
  float pdf;
  bool delta;
};

// Light.sample (Light.hs:122-160)
static LightSample lightSample(const orc_scene& S, const Light& l, V p, float eps, V n, float u1,
                               float u2) {
  LightSample ls;
  if (l.kind == LIGHT_AREA) {
    const Shape& s = S.shapes[l.shape];
    V pl = transPoint(s.o2w.i, p);  // w2l
    V ps, ns;
    sampleShape(s, pl, u1, u2, ps, ns);
    V wi = normalize(ps - pl);
    ls.li = dot(ns, wi) < 0 ? s.emission : BLACK;
    ls.wi = transVector(s.o2w.m, wi);
    ls.pdf = shapePdf(s, pl, wi);
    Ray rl{pl, wi, eps, len(ps - pl) - eps};
    ls.ray = transRay(s.o2w.m, rl);
    ls.delta = false;
    return ls;
  }
  if (l.kind == BLING_LIGHT_DIRECTIONAL) {
    ls.li = sScale(l.spec, absDot(n, l.vec));
    ls.wi = l.vec;
    ls.ray = Ray{p, l.vec, eps, INF};
    ls.pdf = 1;
    ls.delta = true;
    return ls;
  }
  if (l.kind == BLING_LIGHT_POINT) {
    ls.li = sScale(l.spec, 1.0f / sqLen(l.vec - p));
    ls.wi = normalize(l.vec - p);
    ls.ray = Ray{p, l.vec - p, eps, INF};
    ls.pdf = 1;
    ls.delta = true;
    return ls;
  }
  // infinite (Light.hs:130-141)
  float v, pdf1, u, pdf0;
  int im, iu;
  sampleContinuous1D(l.mfunc, l.mcdf, l.mint, u2, v, pdf1, im);
  sampleContinuous1D(l.cfunc[im], l.ccdf[im], l.cint[im], u1, u, pdf0, iu);
  float mapPdf = pdf0 * pdf1;
  LightSample none{BLACK, V{0, 1, 0}, Ray{V{0, 0, 0}, V{0, 1, 0}, 0, 1}, 0, false};
  if (mapPdf == 0) return none;
  float phi = u * 2.0f * PI, theta = v * PI;  // cartToSph
  float sint = sinf(theta);
  if (sint == 0) return none;
  ls.li = envLookup(l, u, v);
  V dl = sphericalDirection(sinf(theta), cosf(theta), phi);
  ls.wi = transVector(l.w2l.i, dl);  // inverse w2l
  ls.ray = Ray{p, ls.wi, eps, INF};
  ls.pdf = mapPdf / (2.0f * PI * PI * sint);
  ls.delta = false;
  return ls;
}
// Light.le (Light.hs:98-106)
static Spec lightLe(const Light& l, const Ray& r) {
  if (l.kind != BLING_LIGHT_INFINITE) return BLACK;
  V wh = normalize(transVector(l.w2l.m, r.d));
  float phi = sphericalPhi(wh), theta = sphericalTheta(wh);
  return envLookup(l, phi / (2.0f * PI), theta / PI);  // sphToCart
}
// Light.pdf (Light.hs:215-229)
static float lightPdf(const orc_scene& S, const Light& l, V p, V wi) {
  if (l.kind == LIGHT_AREA) {
    const Shape& s = S.shapes[l.shape];
    return shapePdf(s, transPoint(s.o2w.i, p), transVector(s.o2w.i, wi));
  }
  if (l.kind != BLING_LIGHT_INFINITE) return 0;
  V d = transVector(l.w2l.m, wi);
  float theta = sphericalTheta(d), phi = sphericalPhi(d);
  float sint = sinf(theta);
  if (sint == 0) return 0;
  float u = phi / (2.0f * PI), v = theta / PI;
  // pdfDist2D (Montecarlo.hs:95-106)
  int nu = (int)l.cfunc[0].size(), nv = (int)l.mfunc.size();
  int iu = std::max(0, std::min(nu - 1, (int)floorf(u * (float)nu)));
  int iv = std::max(0, std::min(nv - 1, (int)floorf(v * (float)nv)));
  float pd;
  if (l.mint * l.cint[iv] == 0)
    pd = 0;
  else
    pd = (l.cfunc[iv][iu] * l.mfunc[iv]) / (l.cint[iv] * l.mint);
  return pd / (2.0f * PI * PI * sint);
}

// ---------------------------------------------------------------- integrator
struct Counters {
  uint64_t closest = 0, any = 0;
};

// intLe (Primitive.hs:68-76) + lEmit (Light.hs:85-96)
static Spec intLe(const orc_scene& S, const Isect& it, V wo) {
  const Prim& pr = S.prims[it.prim];
  if (!pr.is_shape) return BLACK;
  const Shape& s = S.shapes[pr.index];
  if (!s.emissive) return BLACK;
  return dot(it.dg.n, wo) > 0 ? s.emission : BLACK;
}
static int intLightId(const orc_scene& S, const Isect& it) {
  const Prim& pr = S.prims[it.prim];
  if (!pr.is_shape) return -1;
  const Shape& s = S.shapes[pr.index];
  return s.emissive ? s.light_id : -1;
}

// Ray counts of the MIS ray, as the GPU integrator queries it (the answer
// is the same either way; this only sets which counter it goes to): an
// any-hit query up to the light toward an area light whose shape the ray
// meets, an any-hit query toward an infinite light, and none otherwise when
// the term is zero whatever the ray meets (an area light it misses or a
// point or directional light: le is zero; f and the weight finite, the ray
// without NaN), else an any-hit query.
static void countMisRay(const orc_scene& S, const Light& l, V p, const BsdfSample& b,
                        const Ray& ray, Counters& C) {
  if (l.kind == LIGHT_AREA) {
    const Shape& s = S.shapes[l.shape];
    float t, e;
    DG dg;
    if (shapeIntersect(s, transRay(s.o2w.i, ray), t, e, dg)) {
      C.any++;
      return;
    }
  }
  bool finite = std::isfinite(powerHeuristic(b.pdf, lightPdf(S, l, p, b.wi)));
  for (int i = 0; i < 16; i++) finite = finite && std::isfinite(b.f.v[i]);
  bool nan_ray = std::isnan(ray.o.x) || std::isnan(ray.o.y) || std::isnan(ray.o.z) ||
                 std::isnan(ray.d.x) || std::isnan(ray.d.y) || std::isnan(ray.d.z) ||
                 std::isnan(ray.tmin) || std::isnan(ray.tmax);
  if (l.kind == BLING_LIGHT_INFINITE || !finite || nan_ray) C.any++;
}

// estimateDirect = sampleLightMis + sampleBsdfMis (Scene.hs:61-99)
static Spec estimateDirect(const orc_scene& S, int li, V p, float eps, V n, V wo, const Bsdf& bsdf,
                           float ld1, float ld2, float ubc, float ubd1, float ubd2, Counters& C) {
  const Light& l = S.lights[li];
  Spec ls = BLACK;
  {
    LightSample smp = lightSample(S, l, p, eps, n, ld1, ld2);
    if (!(smp.pdf == 0 || isBlack(smp.li))) {
      Spec f = evalBsdf(bsdf, wo, smp.wi);
      if (!isBlack(f)) {
        C.any++;
        if (!occluded(S, smp.ray)) {
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
  Spec bs = BLACK;
  {
    BsdfSample b = sampleBsdf(bsdf, wo, ubc, ubd1, ubd2);
    if (!(b.pdf == 0 || isBlack(b.f))) {
      Ray ray{p, b.wi, eps, INF};
      Isect hit;
      countMisRay(S, l, p, b, ray, C);
      bool h = sceneIntersect(S, ray, hit);
      auto sc = [&](const Spec& lr) {
        float lPdf = lightPdf(S, l, p, b.wi);
        return sScale(b.f * lr, powerHeuristic(b.pdf, lPdf));
      };
      if (h) {
        int lid = intLightId(S, hit);
        if (lid >= 0 && l.kind == LIGHT_AREA && lid == l.id) bs = sc(intLe(S, hit, -b.wi));
      } else {
        bs = sc(lightLe(l, ray));
      }
    }
  }
  return ls + bs;
}

// Path.hs:41-87, iterated instead of recursed; returns L
static Spec pathLi(const orc_scene& S, const Sampler& smp, Ray ray, int md, int rrDepth,
                   Counters& C) {
  Spec t = WHITE, l = BLACK;
  bool spec = true;
  Isect it;
  C.closest++;
  bool hit = sceneIntersect(S, ray, it);
  for (int depth = 0;; depth++) {
    if (!hit) {
      if (spec) {
        Spec sum = BLACK;
        for (const Light& lt : S.lights) sum = sum + lightLe(lt, ray);
        return l + t * sum;
      }
      return l;
    }
    if (depth == md) return l;
    float lNumU = rnd1(smp, 1 + 4 * depth);
    float ld1, ld2;
    rnd2(smp, 1 + 3 * depth, ld1, ld2);
    float lBsdfCompU = rnd1(smp, 2 + 4 * depth);
    float lb1, lb2;
    rnd2(smp, 2 + 3 * depth, lb1, lb2);
    V rd = ray.d;
    Spec intl = spec ? intLe(S, it, rd) : BLACK;
    V wo = -rd;
    const Prim& pr = S.prims[it.prim];
    int mat = pr.is_shape ? S.shapes[pr.index].material : S.meshes[pr.index].material;
    DG dgs = shadingGeometry(S, pr, it.dg);
    Material mm = hitMaterial(S, mat, it.dg, dgs);
    Bsdf bsdf = materialBsdf(mm, it.dg, dgs);
    V n = bsdf.cs.n;
    V p = bsdf.p;
    float eps = it.eps;
    // sampleOneLight (Scene.hs:109-118)
    Spec direct = BLACK;
    int lc = (int)S.lights.size();
    if (lc == 1) {
      direct = estimateDirect(S, 0, p, eps, n, wo, bsdf, ld1, ld2, lBsdfCompU, lb1, lb2, C);
    } else if (lc > 1) {
      int ln = std::min((int)floorf(lNumU * (float)lc), lc - 1);
      direct = sScale(estimateDirect(S, ln, p, eps, n, wo, bsdf, ld1, ld2, lBsdfCompU, lb1, lb2, C),
                      (float)lc);
    }
    Spec lHere = intl + direct;
    l = l + t * lHere;
    float pc = depth <= rrDepth ? 1.0f : hmin(0.75f, sY(t));
    float x = rnd1(smp, 3 + 4 * depth);
    if (x > pc) return l;
    float uc = rnd1(smp, 0 + 4 * depth);
    float ud1, ud2;
    rnd2(smp, 0 + 3 * depth, ud1, ud2);
    BsdfSample bs = sampleBsdf(bsdf, wo, uc, ud1, ud2);
    if (bs.pdf == 0 || isBlack(bs.f)) return l;
    t = sScale(bs.f * t, 1.0f / pc);
    spec = (bs.type & T_SPEC) != 0;
    ray = Ray{p, bs.wi, eps, INF};
    C.closest++;
    hit = sceneIntersect(S, ray, it);
  }
}

// hash (SPPM.hs:303-305) and the bucket of a cell: abs (hash) `rem` cnt, clamped
static long long cellBucketOf(long long x, long long y, long long z, long long cnt) {
  long long h = (long long)((unsigned long long)x * 73856093ull ^ (unsigned long long)y * 19349663ull ^
                            (unsigned long long)z * 83492791ull);
  h = h < 0 ? -h : h;
  long long r = h % cnt;
  return r < 0 ? 0 : (r > cnt - 1 ? cnt - 1 : r);
}

// ---------------------------------------------------------------- light tracer
// Renderer/LightTracer.hs.  A photon's random numbers come from the shared
// generator keyed by (seed, pass, photon): dimension 0 picks the light, 1-2
// the point on it, 3-4 the direction (oneRay, LightTracer.hs:46-55); vertex d
// draws 5+4d (BSDF component), 6+4d and 7+4d (direction) and 8+4d (Russian
// roulette) (nextVertex, LightTracer.hs:81-110).
static inline uint64_t photonKey(uint64_t seed, uint64_t pass, uint64_t photon) {
  return pixelKey(seed, pass, -0x4c54, (int)(uint32_t)(photon >> 32));
}

// sample' (Light.hs:166-213): the emitted radiance, the ray leaving the
// light, the normal there and the pdf; (wc, wr) is the bounding sphere of the
// scene (boundingSphere, AABB.hs:62-66)
static void lightEmit(const orc_scene& S, const Light& l, V wc, float wr, float uo1, float uo2,
                      float ud1, float ud2, Spec& r, Ray& ray, V& ns, float& pd) {
  if (l.kind == LIGHT_AREA) {
    const Shape& s = S.shapes[l.shape];
    V orgp, nsp;
    sampleShapeP(s, uo1, uo2, orgp, nsp);  // sampleShape'
    V org = transPoint(s.o2w.m, orgp);
    ns = normalize(transNormal(s.o2w.i, nsp));
    V wi = localToWorld(coordinateSystem(ns), cosineSampleHemisphere(ud1, ud2));
    pd = INV_PI * (1.0f / shapeArea(s)) * absDot(ns, wi);  // shapePdf' = 1 / area
    ray = Ray{org, wi, 1e-3f, INF};
    r = s.emission;
    return;
  }
  if (l.kind == BLING_LIGHT_DIRECTIONAL) {
    LC c = coordinateSystem(l.vec);  // coordinateSystem''
    float d1, d2;
    concentricSampleDisk(uo1, uo2, d1, d2);
    V pdisk = wc + sv(wr, sv(d1, c.s) + sv(d2, c.t));
    ns = -l.vec;
    ray = Ray{pdisk + sv(wr, l.vec), ns, 0, INF};
    pd = 1.0f / (PI * wr * wr);
    r = l.spec;
    return;
  }
  if (l.kind == BLING_LIGHT_POINT) {
    V d = uniformSampleSphere(ud1, ud2);
    ray = Ray{l.vec, d, 0, INF};
    pd = 1.0f / (2.0f * PI);  // uniformSpherePdf (Montecarlo.hs:188-190)
    ns = d;
    r = l.spec;
    return;
  }
  // infinite: sampleContinuous2D over the map, then a disk across the scene
  float v, pdf1, u, pdf0;
  int im, iu;
  sampleContinuous1D(l.mfunc, l.mcdf, l.mint, ud2, v, pdf1, im);
  sampleContinuous1D(l.cfunc[im], l.ccdf[im], l.cint[im], ud1, u, pdf0, iu);
  float mapPdf = pdf0 * pdf1;
  if (mapPdf == 0) {  // emptySample'
    r = BLACK;
    ray = Ray{V{0, 0, 0}, V{0, 1, 0}, 0, 0};
    ns = V{0, 1, 0};
    pd = 0;
    return;
  }
  r = envLookup(l, u, v);
  float phi = u * 2.0f * PI, theta = v * PI;  // cartToSph
  V d = transVector(l.w2l.i, sphericalDirection(sinf(theta), cosf(theta), phi));
  LC c = coordinateSystem(-d);
  float d1, d2;
  concentricSampleDisk(uo1, uo2, d1, d2);
  V pDisk = wc + sv(wr, sv(d1, c.s) + sv(d2, c.t));
  ray = Ray{pDisk + sv(wr, d), -d, 0, INF};
  float sint = sinf(theta);
  float pdDir = mapPdf / (2.0f * PI * PI * sint);
  float pdArea = 1.0f / (PI * wr * wr);
  pd = sint == 0 ? 0.0f : pdDir * pdArea;
  ns = d;
}

// sampleCam of the projective camera (Camera.hs:90-100): the raster
// position of world point p, the lens centre and the pdf
static void sampleCam(const bling_camera_desc& cam, V p, float& px, float& py, V& pLens,
                      float& cPdf) {
  V pRas = transPoint(cam.w2r, p);
  pLens = transPoint(cam.c2w, V{0, 0, 0});
  float cost = fabsf(normalize(transPoint(cam.r2c, pRas)).z);
  float cost3 = cost * cost * cost;
  cPdf = cam.pixel_area * cost3;
  px = pRas.x;
  py = pRas.y;
}

struct SplatImg {  // the splat part of MImage (Image.hs:64-71), origin (0, 0)
  int w, h;
  float* xyz;
  uint64_t splats = 0, nonfinite = 0;
};

// connectCam (LightTracer.hs:57-71) with splatSample (Image.hs:201-221).  A
// splat outside the image is dropped before its visibility is asked (the
// reference asks first; the image is the same).
static void connectCam(const orc_scene& S, SplatImg& img, const Spec& li, const Bsdf& bsdf, V wi,
                       float eps, Counters& C) {
  float px, py, cPdf;
  V pCam;
  V p = bsdf.p;
  sampleCam(S.cam, p, px, py, pCam, cPdf);
  V dCam = pCam - p;
  V we = normalize(dCam);
  Spec f = evalBsdf(bsdf, wi, we, true);
  if (isBlack(f) || cPdf == 0) return;
  float dCam2 = sqLen(dCam);
  Spec lr = sScale(li * f, 1.0f / (cPdf * dCam2));
  if (!(px >= 0.0f && px < (float)img.w && py >= 0.0f && py < (float)img.h)) return;
  C.any++;
  if (occluded(S, Ray{p, we, eps, sqrtf(dCam2)})) return;
  if (sNaN(lr) || sInf(lr)) {
    img.nonfinite++;
    return;
  }
  int ix = (int)floorf(px), iy = (int)floorf(py);
  float x, y, z;
  spectrumToXYZ(lr, x, y, z);
  float* o = img.xyz + 3 * ((size_t)iy * img.w + ix);
  o[0] = o[0] + x;
  o[1] = o[1] + y;
  o[2] = o[2] + z;
  img.splats++;
}

// oneRay + nextVertex (LightTracer.hs:46-110) for photon g, iterated;
// max_depth > 0 stops a photon after that many vertices
static void tracePhoton(const orc_scene& S, uint64_t seed, uint64_t pass, uint64_t g, V wc,
                        float wr, int max_depth, SplatImg& img, Counters& C) {
  uint64_t key = photonKey(seed, pass, g);
  uint32_t n = (uint32_t)g;
  int lc = (int)S.lights.size();
  if (lc == 0) return;  // sampleLightRay of no lights: pdf 0
  float ul = randF(key, n, 0);
  float uo1 = randF(key, n, 1), uo2 = randF(key, n, 2);
  float ud1 = randF(key, n, 3), ud2 = randF(key, n, 4);
  int ln = lc == 1 ? 0 : std::min((int)floorf(ul * (float)lc), lc - 1);
  Spec le;
  Ray ray;
  V nl;
  float pdf;
  lightEmit(S, S.lights[ln], wc, wr, uo1, uo2, ud1, ud2, le, ray, nl, pdf);
  if (lc != 1) pdf = pdf / (float)lc;  // sampleLightRay (Scene.hs:121-135)
  V wo = normalize(ray.d);
  Spec li = sScale(le, absDot(nl, wo) / pdf);
  if (!(pdf > 0 && !isBlack(li))) return;
  V wi = -wo;
  Isect it;
  C.closest++;
  bool hit = sceneIntersect(S, ray, it);
  for (int depth = 0;; depth++) {
    if (!hit || isBlack(li)) return;
    uint32_t dim = 5 + 4 * (uint32_t)depth;
    float ubc = randF(key, n, dim), ubd1 = randF(key, n, dim + 1), ubd2 = randF(key, n, dim + 2);
    float pcont = depth > 3 ? 0.8f : 1.0f;
    const Prim& pr = S.prims[it.prim];
    int mat = pr.is_shape ? S.shapes[pr.index].material : S.meshes[pr.index].material;
    DG dgs = shadingGeometry(S, pr, it.dg);
    Material mm = hitMaterial(S, mat, it.dg, dgs);
    Bsdf bsdf = materialBsdf(mm, it.dg, dgs);
    V p = bsdf.p;
    BsdfSample bs = sampleBsdf(bsdf, wi, ubc, ubd1, ubd2, true);  // sampleAdjBsdf
    Spec li2 = sScale(li * bs.f, 1.0f / pcont);
    connectCam(S, img, li, bsdf, wi, it.eps, C);
    if (isBlack(bs.f) || bs.pdf == 0) return;
    if (randF(key, n, dim + 3) > pcont) return;
    if (max_depth > 0 && depth + 1 >= max_depth) return;
    ray = Ray{p, bs.wi, it.eps, INF};
    C.closest++;
    hit = sceneIntersect(S, ray, it);
    wi = -bs.wi;
    li = li2;
  }
}

// ---------------------------------------------------------------- film
// evalFilter (Filter.hs:68-96)
static float evalFilter(int kind, const float* fp, float x, float y) {
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
        float xp = fabsf(xx) * PI;
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
static void filterSize(int kind, const float* fp, float& fw, float& fh) {
  if (kind == BLING_FILTER_BOX) {
    fw = fh = 0.5f;
  } else {
    fw = fp[0];
    fh = fp[1];
  }
}
// mkTableFilter (Image.hs:48-61)
static void filterTable(int kind, const float* fp, float* out) {
  float fw, fh;
  filterSize(kind, fp, fw, fh);
  for (int y = 0; y < 16; y++) {
    float fy = ((float)y + 0.5f) * fh / 16.0f;
    for (int x = 0; x < 16; x++) {
      float fx = ((float)x + 0.5f) * fw / 16.0f;
      out[y * 16 + x] = evalFilter(kind, fp, fx, fy);
    }
  }
}

// The pixel sums are binary32 as in the reference (T = float), or binary64
// (T = double) for reference renders with many samples per pixel: each
// binary32 product w * XYZ is then added in double precision.
template <class T>
struct FilmImg {  // MImage (Image.hs:64-71), pixel part
  int w, h, ox, oy;
  T* p;
};
// addSample (Image.hs:250-299); returns false when dropped as NaN/Inf
template <class T>
static bool addSample(FilmImg<T>& img, const float* tblv, float fw, float fh, float sx, float sy,
                      const Spec& ss) {
  if (sNaN(ss) || sInf(ss)) return false;
  float smx, smy, smz;
  spectrumToXYZ(ss, smx, smy, smz);
  float ifw = 1.0f / fw, ifh = 1.0f / fw;  // sic (Image.hs:263)
  float dx = sx - 0.5f, dy = sy - 0.5f;
  int x0 = std::max(img.ox, (int)ceilf(dx - fw));
  int x1 = std::min(img.ox + img.w - 1, (int)floorf(dx + fw));
  int y0 = std::max(img.oy, (int)ceilf(dy - fh));
  int y1 = std::min(img.oy + img.h - 1, (int)floorf(dy + fh));
  if (x1 - x0 < 0 || y1 - y0 < 0) return true;
  for (int y = y0; y <= y1; y++) {
    float fy = fabsf(((float)y - dy) * ifh * 16.0f);
    int iy = std::min((int)floorf(fy), 15);
    for (int x = x0; x <= x1; x++) {
      float fx = fabsf(((float)x - dx) * ifw * 16.0f);
      int ix = std::min((int)floorf(fx), 15);
      float w = tblv[iy * 16 + ix];
      T* px = img.p + 4 * ((size_t)(x - img.ox) + (size_t)(y - img.oy) * img.w);
      px[0] = px[0] + (T)w;
      px[1] = px[1] + (T)(smx * w);
      px[2] = px[2] + (T)(smy * w);
      px[3] = px[3] + (T)(smz * w);
    }
  }
  return true;
}

static int nthreadsOf(int n) {
  if (n > 0) return n;
  unsigned h = std::thread::hardware_concurrency();
  return h ? (int)h : 1;
}
template <class F>
static void parallelFor(size_t n, int nth, F f) {
  nth = nthreadsOf(nth);
  if (nth <= 1 || n < 64) {
    for (size_t i = 0; i < n; i++) f(i);
    return;
  }
  std::atomic<size_t> next{0};
  std::vector<std::thread> ts;
  for (int k = 0; k < nth; k++)
    ts.emplace_back([&]() {
      for (;;) {
        size_t b = next.fetch_add(256);
        if (b >= n) break;
        size_t e = std::min(n, b + 256);
        for (size_t i = b; i < e; i++) f(i);
      }
    });
  for (auto& t : ts) t.join();
}

static Ray rayOf(const float* rays, size_t n, size_t i) {
  return Ray{V{rays[i], rays[n + i], rays[2 * n + i]}, V{rays[3 * n + i], rays[4 * n + i], rays[5 * n + i]},
             rays[6 * n + i], rays[7 * n + i]};
}

// ---------------------------------------------------------------- transforms
// the matrix algebra of Transform.hs:44-110
static void mmul(const float* m1, const float* m2, float* out) {  // mul m1 m2 (Transform.hs:102-105)
  for (int n = 0; n < 16; n++) {
    int i = n / 4, j = n % 4;
    float s = 0.0f;
    for (int k = 0; k < 4; k++) s = s + m1[k * 4 + j] * m2[i * 4 + k];
    out[n] = s;
  }
}
static void minvert(const float* m, float* out) {  // invert (Transform.hs:44-87)
  float a[16];
  memcpy(a, m, sizeof a);
  auto idx = [](int r, int c) { return c * 4 + r; };
  std::vector<int> ipiv = {0, 1, 2, 3};
  int indx_r[4], indx_c[4];
  for (int step = 0; step < 4; step++) {
    int irow = -1, icol = -1;
    float best = 0;
    bool first = true;
    for (int j : ipiv)
      for (int k : ipiv) {
        // maximumBy (compare `on` abs): a later element wins unless strictly smaller
        float v = fabsf(a[idx(j, k)]);
        if (first || best < v || best == v) {
          best = v;
          irow = j;
          icol = k;
        }
        first = false;
      }
    ipiv.erase(std::remove(ipiv.begin(), ipiv.end(), icol), ipiv.end());
    if (irow != icol)
      for (int k = 0; k < 4; k++) std::swap(a[idx(irow, k)], a[idx(icol, k)]);
    float pivinv = 1.0f / a[idx(icol, icol)];
    a[idx(icol, icol)] = 1.0f;
    for (int j = 0; j < 4; j++) a[idx(icol, j)] = a[idx(icol, j)] * pivinv;
    for (int j = 0; j < 4; j++) {
      if (j == icol) continue;
      float save = a[idx(j, icol)];
      a[idx(j, icol)] = 0.0f;
      for (int k = 0; k < 4; k++) {
        float x = a[idx(icol, k)];
        float old = a[idx(j, k)];
        a[idx(j, k)] = old - x * save;
      }
    }
    indx_r[step] = irow;
    indx_c[step] = icol;
  }
  for (int s = 3; s >= 0; s--) {
    int ir = indx_r[s], ic = indx_c[s];
    if (ir != ic)
      for (int k = 0; k < 4; k++) std::swap(a[idx(k, ir)], a[idx(k, ic)]);
  }
  memcpy(out, a, sizeof a);
}
static void setm(float* m, float a, float b, float c, float d, float e, float f, float g, float h,
                 float i, float j, float k, float l, float mm, float n, float o, float p) {
  float v[16] = {a, b, c, d, e, f, g, h, i, j, k, l, mm, n, o, p};
  memcpy(m, v, sizeof v);
}

}  // namespace

// ================================================================ C API
extern "C" {

int orc_scene_create(const bling_scene_desc* d, orc_scene** out) {
  if (!d || !out) return BLING_ERR_INVALID_ARG;
  orc_scene* S = new orc_scene();
  for (int i = 0; i < d->n_materials; i++) {
    const bling_material& bm = d->materials[i];
    Material m;
    m.kind = bm.kind;
    m.sigma = bm.sigma;
    m.rough = bm.roughness;
    m.ior = bm.ior;
    memcpy(m.kd.v, bm.kd, 64);
    memcpy(m.ks.v, bm.ks, 64);
    memcpy(m.kt.v, bm.kt, 64);
    memcpy(m.eta.v, bm.eta, 64);
    memcpy(m.k.v, bm.k, 64);
    m.kd_tex = bm.kd_texture;
    memcpy(m.kd_par, bm.kd_tex_params, 36);
    memcpy(m.kd2.v, bm.kd2, 64);
    memcpy(m.tex, bm.tex, sizeof m.tex);
    m.bump = bm.bump;
    S->mats.push_back(m);
  }
  for (int i = 0; i < d->n_textures; i++) {
    const bling_texture& t = d->textures[i];
    TexNode n;
    n.kind = t.kind;
    n.a = t.a;
    n.b = t.b;
    n.c = t.c;
    n.ivalue = t.ivalue;
    n.map_kind = t.map_kind;
    memcpy(n.map, t.map, 64);
    memcpy(n.p, t.p, 16);
    memcpy(n.spectrum.v, t.spectrum, 64);
    n.w = t.width;
    n.h = t.height;
    if (t.kind == BLING_TEXN_GRADIENT) {
      // mkGradient: sortBy (compare `on` fst), a stable sort (Texture.hs:228-234)
      std::vector<std::pair<float, int>> key;
      for (int k = 0; k < t.ivalue; k++) key.push_back({t.data[17 * k], k});
      std::stable_sort(key.begin(), key.end(),
                       [](const std::pair<float, int>& x, const std::pair<float, int>& y) {
                         return x.first < y.first;
                       });
      for (auto& kv : key) n.steps.insert(n.steps.end(), t.data + 17 * kv.second, t.data + 17 * kv.second + 17);
    }
    if (t.kind == BLING_TEXN_IMAGE) n.pixels.assign(t.pixels, t.pixels + (size_t)3 * t.width * t.height);
    if (t.kind == BLING_TEXN_IMAGE_SCALAR) n.pixels.assign(t.pixels, t.pixels + (size_t)t.width * t.height);
    S->tex.push_back(std::move(n));
  }
  for (int i = 0; i < d->n_meshes; i++) {
    const bling_mesh_desc& md = d->meshes[i];
    Mesh m;
    if (md.n_indices % 3 != 0) {
      delete S;
      return BLING_ERR_INVALID_ARG;
    }
    m.p.resize(md.n_vertices);
    for (int64_t k = 0; k < md.n_vertices; k++)
      m.p[k] = V{md.vertices[3 * k], md.vertices[3 * k + 1], md.vertices[3 * k + 2]};
    m.idx.assign(md.indices, md.indices + md.n_indices);
    for (int32_t v : m.idx)
      if (v < 0 || v >= md.n_vertices) {
        delete S;
        return BLING_ERR_INVALID_ARG;
      }
    if (md.normals) {
      m.n.resize(md.n_vertices);
      for (int64_t k = 0; k < md.n_vertices; k++)
        m.n[k] = V{md.normals[3 * k], md.normals[3 * k + 1], md.normals[3 * k + 2]};
    }
    if (md.uvs) m.uv.assign(md.uvs, md.uvs + 2 * md.n_vertices);
    m.material = md.material;
    S->meshes.push_back(std::move(m));
  }
  for (int i = 0; i < d->n_shapes; i++) {
    const bling_shape_desc& sd = d->shapes[i];
    Shape s;
    s.kind = sd.kind;
    memcpy(s.p, sd.params, sizeof s.p);
    memcpy(s.o2w.m, sd.o2w, 64);
    memcpy(s.o2w.i, sd.w2o, 64);
    s.material = sd.material;
    s.emissive = sd.emissive != 0;
    memcpy(s.emission.v, sd.emission, 64);
    s.light_id = -1;
    S->shapes.push_back(s);
  }
  // user lights first (Scene.hs:39)
  for (int i = 0; i < d->n_lights; i++) {
    const bling_light_desc& ld = d->lights[i];
    Light l;
    l.kind = ld.kind;
    memcpy(l.spec.v, ld.spectrum, 64);
    l.vec = V{ld.vec[0], ld.vec[1], ld.vec[2]};
    l.shape = -1;
    l.id = -1;
    l.w = l.h = 0;
    l.sky = false;
    if (ld.kind == BLING_LIGHT_INFINITE || ld.kind == BLING_LIGHT_SUNSKY) {
      if (ld.kind == BLING_LIGHT_SUNSKY) {  // mkDiscreteTextureMap2d (640, 480) eval
        l.kind = BLING_LIGHT_INFINITE;
        l.sky = true;
        l.skyd = initSkyData(mkV(ld.east[0], ld.east[1], ld.east[2]), l.vec, ld.turbidity);
        l.w = 640;
        l.h = 480;
      } else {
        l.w = ld.env_w;
        l.h = ld.env_h;
        l.env.resize((size_t)l.w * l.h);
        for (size_t k = 0; k < l.env.size(); k++) memcpy(l.env[k].v, ld.env + 16 * k, 64);
      }
      memcpy(l.w2l.m, ld.w2l, 64);
      memcpy(l.w2l.i, ld.l2w, 64);
      // mkInfiniteAreaLight: dist = mkDist2D (texSize) (sY . eval) (Light.hs:76-82)
      l.cfunc.resize(l.h);
      l.ccdf.resize(l.h);
      l.cint.resize(l.h);
      for (int v = 0; v < l.h; v++) {
        l.cfunc[v].resize(l.w);
        for (int u = 0; u < l.w; u++)
          l.cfunc[v][u] = sY(envLookup(l, (float)u / (float)l.w, (float)v / (float)l.h));
        mkDist1D(l.cfunc[v], l.ccdf[v], l.cint[v]);
      }
      l.mfunc = l.cint;
      mkDist1D(l.mfunc, l.mcdf, l.mint);
    }
    S->lights.push_back(std::move(l));
  }
  // primitive list
  std::vector<int32_t> order;
  if (d->prim_order) {
    order.assign(d->prim_order, d->prim_order + d->n_meshes + d->n_shapes);
  } else {
    for (int i = 0; i < d->n_meshes; i++) order.push_back(i);
    for (int i = 0; i < d->n_shapes; i++) order.push_back(~i);
  }
  for (int32_t v : order) {
    if (v >= 0) {
      const Mesh& m = S->meshes[v];
      for (size_t t = 0; t < m.idx.size() / 3; t++) {
        Prim p;
        p.is_shape = 0;
        p.index = v;
        p.tri = (int)t;
        p.p1 = m.p[m.idx[3 * t]];
        p.p2 = m.p[m.idx[3 * t + 1]];
        p.p3 = m.p[m.idx[3 * t + 2]];
        S->prims.push_back(p);
      }
    } else {
      Prim p{};
      p.is_shape = 1;
      p.index = ~v;
      S->prims.push_back(p);
      Shape& s = S->shapes[~v];
      if (s.emissive) {  // geometric lights in primitive order (Scene.hs:42)
        Light l;
        l.kind = LIGHT_AREA;
        l.shape = ~v;
        l.id = (int)S->lights.size();
        s.light_id = l.id;
        l.w = l.h = 0;
        S->lights.push_back(std::move(l));
      }
    }
  }
  S->cam = d->camera;
  buildOracleBvh(*S);
  *out = S;
  return BLING_OK;
}

void orc_scene_destroy(orc_scene* s) { delete s; }
int64_t orc_scene_prim_count(const orc_scene* s) { return (int64_t)s->prims.size(); }

void orc_trace_closest_brute(const orc_scene* s, const float* rays, size_t n, float* t,
                             int32_t* prim, float* b1b2, int nth) {
  parallelFor(n, nth, [&](size_t i) {
    Hit h;
    Ray r = rayOf(rays, n, i);
    if (closestBrute(*s, r, h)) {
      t[i] = h.t;
      prim[i] = h.prim;
      if (b1b2) {
        b1b2[2 * i] = h.b1;
        b1b2[2 * i + 1] = h.b2;
      }
    } else {
      t[i] = INF;
      prim[i] = -1;
      if (b1b2) b1b2[2 * i] = b1b2[2 * i + 1] = 0;
    }
  });
}
void orc_trace_any_brute(const orc_scene* s, const float* rays, size_t n, uint8_t* hit, int nth) {
  parallelFor(n, nth, [&](size_t i) { hit[i] = anyBrute(*s, rayOf(rays, n, i)) ? 1 : 0; });
}
void orc_trace_closest_bvh(const orc_scene* s, const float* rays, size_t n, float* t,
                           int32_t* prim, float* b1b2, int nth) {
  parallelFor(n, nth, [&](size_t i) {
    Hit h;
    Ray r = rayOf(rays, n, i);
    if (closestBvh(*s, r, h)) {
      t[i] = h.t;
      prim[i] = h.prim;
      if (b1b2) {
        b1b2[2 * i] = h.b1;
        b1b2[2 * i + 1] = h.b2;
      }
    } else {
      t[i] = INF;
      prim[i] = -1;
      if (b1b2) b1b2[2 * i] = b1b2[2 * i + 1] = 0;
    }
  });
}
void orc_trace_any_bvh(const orc_scene* s, const float* rays, size_t n, uint8_t* hit, int nth) {
  parallelFor(n, nth, [&](size_t i) { hit[i] = anyBvh(*s, rayOf(rays, n, i)) ? 1 : 0; });
}

int orc_kdtree_build(orc_scene* s, int nth, int64_t* stats) {
  if (!s) return BLING_ERR_INVALID_ARG;
  if (!s->kd_built) buildKd(*s, nth > 0 ? nth : nthreadsOf(1 << 30));
  if (stats) {
    const kd::Stats& k = s->kd.stats;
    int64_t v[8] = {k.interiors, k.leaves, k.empty_leaves, k.leaf_refs,
                    k.max_leaf,  k.max_depth, k.depth_sum, s->kd.depth_limit};
    memcpy(stats, v, sizeof v);
  }
  return BLING_OK;
}

int orc_scene_use_kdtree(orc_scene* s, int on, int nth) {
  if (!s) return BLING_ERR_INVALID_ARG;
  if (on && !s->kd_built) orc_kdtree_build(s, nth, nullptr);
  s->use_kd = on != 0;
  return BLING_OK;
}

int orc_trace_closest_kd(orc_scene* s, const float* rays, size_t n, float* t, int32_t* prim,
                         float* b1b2, int nth, uint64_t* counts) {
  if (!s) return BLING_ERR_INVALID_ARG;
  if (!s->kd_built) orc_kdtree_build(s, nth, nullptr);
  std::atomic<uint64_t> nodes{0}, prims{0};
  parallelFor(n, nth, [&](size_t i) {
    Hit h;
    kd::Counts c;
    Ray r = rayOf(rays, n, i);
    if (closestKd(*s, r, h, c)) {
      t[i] = h.t;
      prim[i] = h.prim;
      if (b1b2) {
        b1b2[2 * i] = h.b1;
        b1b2[2 * i + 1] = h.b2;
      }
    } else {
      t[i] = INF;
      prim[i] = -1;
      if (b1b2) b1b2[2 * i] = b1b2[2 * i + 1] = 0;
    }
    if (counts) {
      nodes.fetch_add((uint64_t)c.nodes, std::memory_order_relaxed);
      prims.fetch_add((uint64_t)c.prims, std::memory_order_relaxed);
    }
  });
  if (counts) {
    counts[0] = nodes.load();
    counts[1] = prims.load();
  }
  return BLING_OK;
}

int orc_trace_any_kd(orc_scene* s, const float* rays, size_t n, uint8_t* hit, int nth,
                     uint64_t* counts) {
  if (!s) return BLING_ERR_INVALID_ARG;
  if (!s->kd_built) orc_kdtree_build(s, nth, nullptr);
  std::atomic<uint64_t> nodes{0}, prims{0};
  parallelFor(n, nth, [&](size_t i) {
    kd::Counts c;
    hit[i] = anyKd(*s, rayOf(rays, n, i), c) ? 1 : 0;
    if (counts) {
      nodes.fetch_add((uint64_t)c.nodes, std::memory_order_relaxed);
      prims.fetch_add((uint64_t)c.prims, std::memory_order_relaxed);
    }
  });
  if (counts) {
    counts[0] = nodes.load();
    counts[1] = prims.load();
  }
  return BLING_OK;
}

// sample extent (imageWindow', Image.hs:170-176)
static void sampleExtent(const bling_render_params* p, int& x0, int& x1, int& y0, int& y1) {
  float fw, fh;
  filterSize(p->filter_kind, p->filter_params, fw, fh);
  x0 = (int)floorf(0.5f - fw);
  x1 = (int)floorf(0.5f + (float)p->width + fw);
  y0 = (int)floorf(0.5f - fh);
  y1 = (int)floorf(0.5f + (float)p->height + fh);
}

// camera ray of one sample (fireRay, Camera.hs:49-68)
static Ray cameraRay(const orc_scene* S, float ix, float iy, float lu, float lv) {
  const bling_camera_desc& c = S->cam;
  V pCamera = transPoint(c.r2c, V{ix, iy, 0});
  Ray ray{V{0, 0, 0}, normalize(pCamera), 0, INF};
  if (c.lens_radius > 0) {
    float u, v;
    concentricSampleDisk(lu, lv, u, v);
    V ro{u * c.lens_radius, v * c.lens_radius, 0};
    V pFocus = rayAt(ray, c.focal_distance / ray.d.z);
    ray = Ray{ro, normalize(pFocus - ro), 0, INF};
  }
  return transRay(c.c2w, ray);
}

static Sampler mkSampler(const bling_render_params* p, uint64_t pass, int px, int py, int n) {
  Sampler s;
  s.key = pixelKey(p->seed, pass, px, py);
  s.n = (uint32_t)n;
  s.nu = p->strata_x;
  s.nv = p->strata_y;
  // stratified dimensions (Path.hs:34-36); none for the Random sampler, whose
  // rnd'/rnd2D' always draw fresh uniforms (Sampling.hs:203-221)
  bool random = p->sampler_kind == BLING_SAMPLER_RANDOM;
  s.n1d = random ? 0 : 4 * p->sample_depth;
  s.n2d = random ? 0 : 3 * p->sample_depth;
  return s;
}

static Spec traceSample(const orc_scene* S, const bling_render_params* p, const Sampler& smp,
                        int px, int py, float& sx, float& sy, Counters& C) {
  float ox, oy, lu, lv;
  if (p->sampler_kind == BLING_SAMPLER_RANDOM) {
    // runSample (Random spp): ox, oy, then the lens pair, all uniform
    // (Sampling.hs:101-110)
    ox = randF(smp.key, smp.n, DIM_PIX_U);
    oy = randF(smp.key, smp.n, DIM_PIX_V);
    lu = randF(smp.key, smp.n, DIM_LENS_U);
    lv = randF(smp.key, smp.n, DIM_LENS_V);
  } else {
    strat2D(smp, smp.n, DIM_PIX_U, DIM_PIX_V, ox, oy);  // pixel samples are not shuffled
    uint32_t N = (uint32_t)(p->strata_x * p->strata_y);
    uint32_t lp = permute(smp.n, N, randU32(smp.key, 0xffffffffu, DIM_LENS_PERM));
    strat2D(smp, lp, DIM_LENS_U, DIM_LENS_V, lu, lv);  // lens samples are shuffled
  }
  sx = (float)px + ox;
  sy = (float)py + oy;
  Ray r = cameraRay(S, sx, sy, lu, lv);
  return pathLi(*S, smp, r, p->max_depth, p->rr_depth, C);
}

int orc_sample_li(const orc_scene* s, const bling_render_params* p, uint64_t pass, int px, int py,
                  int n, float* out_xyz, float* out_raster, float* out_spectrum) {
  Counters C;
  Sampler smp = mkSampler(p, pass, px, py, n);
  float sx, sy;
  Spec L = traceSample(s, p, smp, px, py, sx, sy, C);
  spectrumToXYZ(L, out_xyz[0], out_xyz[1], out_xyz[2]);
  out_raster[0] = sx;
  out_raster[1] = sy;
  if (out_spectrum) memcpy(out_spectrum, L.v, 64);
  return BLING_OK;
}

}  // extern "C"

// prender's tiles (Rendering.hs:111-150): every pixel of the sample extent
// gets its samples, each added to its tile's image (mkImageTile, addSample),
// and the tiles are added to the film in order (addTile).  sampleFn(smp, ix,
// iy, tile, sx, sy, C) returns one sample's radiance.
template <class Acc, class SampleFn>
static int renderTiles(const orc_scene* S, const bling_render_params* p, uint64_t pass, Acc* film,
                       int row_begin, int row_end, int nth, int ntiles_hint, SampleFn sampleFn,
                       uint64_t* path_samples, uint64_t* rays_closest, uint64_t* rays_any) {
  (void)S;
  (void)ntiles_hint;
  int x0, x1, y0, y1;
  sampleExtent(p, x0, x1, y0, y1);
  float fw, fh;
  filterSize(p->filter_kind, p->filter_params, fw, fh);
  float tblv[256];
  filterTable(p->filter_kind, p->filter_params, tblv);
  int nsp = p->strata_x * p->strata_y;
  // tiles (splitWindow, Sampling.hs:55-58)
  struct Tile {
    int xs, xe, ys, ye;
  };
  std::vector<Tile> tiles;
  for (int y = y0; y <= y1; y += 16)
    for (int x = x0; x <= x1; x += 16) tiles.push_back(Tile{x, std::min(x + 15, x1), y, std::min(y + 15, y1)});
  int rb = row_begin, re = row_end;
  if (re <= rb) {
    rb = y0;
    re = y1 + 1;
  }
  std::vector<std::vector<Acc>> timgs(tiles.size());
  std::vector<int> tw(tiles.size()), th(tiles.size()), tox(tiles.size()), toy(tiles.size());
  std::atomic<uint64_t> nps{0}, ncl{0}, nany{0};
  parallelFor(tiles.size(), nth, [&](size_t ti) {
    const Tile& T = tiles[ti];
    if (T.ye < rb || T.ys >= re) return;
    // mkImageTile (Image.hs:108-120)
    int px0 = std::max(0, T.xs), py0 = std::max(0, T.ys);
    int w = T.xe - px0 + (int)floorf(0.5f + fw);
    int h = T.ye - py0 + (int)floorf(0.5f + fh);
    tw[ti] = w;
    th[ti] = h;
    tox[ti] = px0;
    toy[ti] = py0;
    Counters C;
    uint64_t ps = 0;
    if (w > 0 && h > 0) timgs[ti].assign((size_t)w * h * 4, (Acc)0);
    FilmImg<Acc> img{w, h, px0, py0, timgs[ti].data()};
    for (int iy = T.ys; iy <= T.ye; iy++) {
      if (iy < rb || iy >= re) continue;
      for (int ix = T.xs; ix <= T.xe; ix++)
        for (int n = 0; n < nsp; n++) {
          Sampler smp = mkSampler(p, pass, ix, iy, n);
          float sx, sy;
          Spec L = sampleFn(smp, ix, iy, ti, sx, sy, C);
          ps++;
          if (w > 0 && h > 0) addSample(img, tblv, fw, fh, sx, sy, L);  // NaN/Inf samples are skipped
        }
    }
    nps += ps;
    ncl += C.closest;
    nany += C.any;
  });
  // addTile in tile order (Rendering.hs:130-134, Image.hs:178-199)
  for (size_t ti = 0; ti < tiles.size(); ti++) {
    if (timgs[ti].empty()) continue;
    int w = tw[ti], h = th[ti], dx = tox[ti], dy = toy[ti];
    for (int y = 0; y < h; y++)
      for (int x = 0; x < w; x++) {
        if (y + dy >= p->height || x + dx >= p->width) continue;
        size_t od = 4 * ((size_t)p->width * (y + dy) + (x + dx));
        size_t os = 4 * ((size_t)w * y + x);
        for (int o = 0; o < 4; o++) film[od + o] = film[od + o] + timgs[ti][os + o];
      }
  }
  if (path_samples) *path_samples = nps;
  if (rays_closest) *rays_closest = ncl;
  if (rays_any) *rays_any = nany;
  return BLING_OK;
}

static size_t extentTiles(const bling_render_params* p) {
  int x0, x1, y0, y1;
  sampleExtent(p, x0, x1, y0, y1);
  return (size_t)((x1 - x0) / 16 + 1) * (size_t)((y1 - y0) / 16 + 1);
}

template <class T>
static int renderPass(const orc_scene* S, const bling_render_params* p, uint64_t pass, T* film,
                      int row_begin, int row_end, int nth, uint64_t* path_samples,
                      uint64_t* rays_closest, uint64_t* rays_any) {
  if (p->strata_x <= 0 || p->strata_y <= 0 || p->width <= 0 || p->height <= 0)
    return BLING_ERR_INVALID_ARG;
  return renderTiles(
      S, p, pass, film, row_begin, row_end, nth, 0,
      [&](const Sampler& smp, int ix, int iy, size_t, float& sx, float& sy, Counters& C) {
        return traceSample(S, p, smp, ix, iy, sx, sy, C);
      },
      path_samples, rays_closest, rays_any);
}
extern "C" {

int orc_render_pass(const orc_scene* S, const bling_render_params* p, uint64_t pass, float* film,
                    int row_begin, int row_end, int nth, uint64_t* path_samples,
                    uint64_t* rays_closest, uint64_t* rays_any) {
  return renderPass(S, p, pass, film, row_begin, row_end, nth, path_samples, rays_closest, rays_any);
}
int orc_render_pass_f64(const orc_scene* S, const bling_render_params* p, uint64_t pass,
                        double* film, int nth, uint64_t* path_samples) {
  return renderPass(S, p, pass, film, 0, 0, nth, path_samples, nullptr, nullptr);
}

}  // extern "C"

// ---------------------------------------------------------------- SPPM
// Renderer/SPPM.hs.  The camera pass's random numbers: the Random sampler's
// pixel and lens dimensions keyed by (seed, 2 pass, pixel), then 3 per node
// of the sample's specular tree, by heap index (root 1, children 2k, 2k+1).
// The photon pass: a stratified sampler with ceil(sqrt n)^2 samples over one
// pixel keyed by (seed, 2 pass + 1, 0, 0), 7 stratified 1D and 5 2D
// dimensions (SPPM.hs:471-474).
static const uint32_t DIM_CAM_TREE = 3u << 20;

// bsdfHasNonSpecular (Reflection.hs:246-249)
static bool bsdfHasNonSpecular(const Bsdf& b) {
  for (int i = 0; i < b.n; i++)
    if (!(b.c[i].type & T_SPEC)) return true;
  return false;
}

// sampleBsdf'' False flags (Reflection.hs:278-316) over the BxDFs whose type
// lies within flags (bxdfMatches)
static BsdfSample sampleBsdfFlags(const Bsdf& b, V woW, int flags, float uComp, float u1, float u2) {
  BsdfSample empty{T_REFL | T_DIFF, 0, BLACK, V{0, 1, 0}};
  int idx[2], cntm = 0;
  for (int i = 0; i < b.n; i++)
    if ((b.c[i].type & flags) == b.c[i].type) idx[cntm++] = i;
  if (cntm == 0) return empty;
  V wo = worldToLocal(b.cs, woW);
  float cntf = (float)cntm;
  float invCnt = 1.0f / cntf;
  int sNum = std::max(0, std::min(cntm - 1, (int)floorf(uComp * cntf)));
  const BxDF& bx = b.c[idx[sNum]];
  Spec fSample;
  V wi;
  float pdfp;
  bxSample(bx, wo, u1, u2, fSample, wi, pdfp);
  V wiW = localToWorld(b.cs, wi);
  float sideTest = dot(wiW, b.ng) / dot(woW, b.ng);
  if (pdfp == 0 || sideTest == 0) return empty;
  bool wantTrans = sideTest < 0;
  auto flt = [&](const BxDF& x) { return wantTrans ? (x.type & T_TRANS) != 0 : (x.type & T_REFL) != 0; };
  if (!flt(bx)) return empty;
  if (bx.type & T_SPEC) return BsdfSample{bx.type, pdfp * invCnt, sScale(fSample, cntf), wiW};
  if (cntm == 1) return BsdfSample{bx.type, pdfp, fSample, wiW};
  float others = 0.0f;
  for (int j = 0; j < cntm; j++)
    if (j != sNum) others = others + bxPdf(b.c[idx[j]], wo, wi);
  float pdf = (pdfp + others) * invCnt;
  Spec fOthers = BLACK;
  for (int j = 0; j < cntm; j++)
    if (j != sNum && flt(b.c[idx[j]])) fOthers = fOthers + bxEval(b.c[idx[j]], wi, wo);
  return BsdfSample{bx.type, pdf, sScale(sScale(fSample, pdfp) + fOthers, 1.0f / pdf), wiW};
}

struct HitPoint {  // HitPoint (SPPM.hs:56-63)
  Bsdf bsdf;
  float px, py, r2;
  V w;
  Spec F;
};

struct PixelStats {  // PixelStats (SPPM.hs:245-262) over the sample extent
  int x0, x1, y0, y1;
  float* r2;
  float* n;
  uint32_t* m;
  int64_t count;
  // sIdx (SPPM.hs:264-274); positions outside the arrays give -1
  int64_t idx(float px, float py) const {
    int w = x1 - x0, h = y1 - y0;
    int ix = std::min(w, (int)px), iy = std::min(h, (int)py);  // truncate
    int64_t i = (int64_t)w * (iy - y0) + (ix - x0);
    return (i >= 0 && i < count) ? i : -1;
  }
};

struct CamTree {
  const orc_scene* S;
  const PixelStats* st;
  uint64_t key;
  uint32_t n;
  int md;
  float sx, sy;
  std::vector<HitPoint>* hps;
  Counters* C;

  // traceCam (SPPM.hs:105-131) of the node with heap index k
  Spec trace(const Ray& ray, int depth, const Spec& t, uint32_t k) {
    if (depth == md) return BLACK;
    Isect it;
    C->closest++;
    if (!sceneIntersect(*S, ray, it)) {
      Spec esc = BLACK;  // escaped (SPPM.hs:74-75)
      for (const Light& l : S->lights) esc = esc + lightLe(l, ray);
      return BLACK + t * esc;
    }
    V wo = -ray.d;
    const Prim& pr = S->prims[it.prim];
    int mat = pr.is_shape ? S->shapes[pr.index].material : S->meshes[pr.index].material;
    DG dgs = shadingGeometry(*S, pr, it.dg);
    Material mm = hitMaterial(*S, mat, it.dg, dgs);
    Bsdf bsdf = materialBsdf(mm, it.dg, dgs);
    Spec ls = t * intLe(*S, it, ray.d);
    if (bsdfHasNonSpecular(bsdf)) {
      int64_t si = st->idx(sx, sy);
      hps->push_back(HitPoint{bsdf, sx, sy, si >= 0 ? st->r2[si] : 0.0f, wo, t});
    }
    Spec lr = follow(T_REFL, it, bsdf, wo, t, depth, k);
    Spec lt = follow(T_TRANS, it, bsdf, wo, t, depth, k);
    return BLACK + lr + lt + ls;
  }
  // followCam (SPPM.hs:89-104)
  Spec follow(int prop, const Isect& it, const Bsdf& bsdf, V wo, const Spec& t, int depth,
              uint32_t k) {
    uint32_t k2 = 2 * k + (prop == T_TRANS ? 1u : 0u);
    uint32_t dim = DIM_CAM_TREE + 3 * k2;
    float uc = randF(key, n, dim), u1 = randF(key, n, dim + 1), u2 = randF(key, n, dim + 2);
    BsdfSample bs = sampleBsdfFlags(bsdf, wo, prop | T_SPEC, uc, u1, u2);
    if (bs.pdf == 0 || isBlack(bs.f)) return BLACK;
    return trace(Ray{bsdf.p, bs.wi, it.eps, INF}, depth + 1, bs.f * t, k2);
  }
};

extern "C" {

int orc_sppm_pass(const orc_scene* S, const bling_sppm_params* sp, int32_t width, int32_t height,
                  uint64_t pass, float* film, float* splat_xyz, float* r2, float* nacc, uint32_t* m,
                  int64_t stat_count, int nth, uint64_t stats[4]) {
  if (width <= 0 || height <= 0 || sp->max_depth < 1 || sp->max_depth > 24) return BLING_ERR_INVALID_ARG;
  bling_render_params rp;
  memset(&rp, 0, sizeof rp);
  rp.width = width;
  rp.height = height;
  rp.strata_x = rp.strata_y = 1;  // mkRandomSampler 1 (SPPM.hs:150)
  rp.max_depth = sp->max_depth;
  rp.rr_depth = 7;
  rp.filter_kind = sp->filter_kind;
  memcpy(rp.filter_params, sp->filter_params, sizeof rp.filter_params);
  rp.seed = sp->seed;
  rp.sampler_kind = BLING_SAMPLER_RANDOM;
  PixelStats st;
  sampleExtent(&rp, st.x0, st.x1, st.y0, st.y1);
  st.count = (int64_t)(st.x1 - st.x0 + 1) * (st.y1 - st.y0 + 1);
  if (stat_count != st.count) return BLING_ERR_BOUNDS;
  st.r2 = r2;
  st.n = nacc;
  st.m = m;
  // ---- camera pass: hit points per tile, in tile order (mkHitPoints, SPPM.hs:133-164)
  std::vector<std::vector<HitPoint>> tile_hps(extentTiles(&rp));
  uint64_t ncam = 0, ncl = 0, nany = 0;
  int rc = renderTiles(
      S, &rp, 2 * pass, film, 0, 0, nth, 0,
      [&](const Sampler& smp, int ix, int iy, size_t tile, float& sx, float& sy, Counters& C) {
        float ox = randF(smp.key, smp.n, DIM_PIX_U), oy = randF(smp.key, smp.n, DIM_PIX_V);
        float lu = randF(smp.key, smp.n, DIM_LENS_U), lv = randF(smp.key, smp.n, DIM_LENS_V);
        sx = (float)ix + ox;
        sy = (float)iy + oy;
        Ray ray = cameraRay(S, sx, sy, lu, lv);
        CamTree tr{S, &st, smp.key, smp.n, sp->max_depth, sx, sy, &tile_hps[tile], &C};
        return tr.trace(ray, 0, WHITE, 1);
      },
      &ncam, &ncl, &nany);
  if (rc) return rc;
  std::vector<HitPoint> hps;
  for (auto& t : tile_hps) hps.insert(hps.end(), t.begin(), t.end());
  uint64_t st_out[4] = {ncl, 0, 0, 0};
  // ---- spatial hash (mkHash, SPPM.hs:297-353); the buckets hold hit-point indices
  int sn = std::max(1, (int)ceilf(sqrtf((float)sp->photons)));
  int64_t nphot = (int64_t)sn * sn;
  long long cnt = (long long)hps.size();
  if (cnt > 0 && !S->lights.empty()) {
    float r2m = 0;
    for (const HitPoint& h : hps) r2m = hmax(h.r2, r2m);
    float r = sqrtf(r2m);
    V lo{INF, INF, INF};
    for (const HitPoint& h : hps) {
      V a = h.bsdf.p - V{r, r, r};
      lo = V{hmin(lo.x, a.x), hmin(lo.y, a.y), hmin(lo.z, a.z)};
    }
    float invSize = 1.0f / (2.0f * r);
    std::vector<std::vector<int>> buckets((size_t)cnt);
    for (long long i = 0; i < cnt; i++) {
      const HitPoint& h = hps[i];
      if (h.r2 == 0) continue;
      float rp = sqrtf(h.r2);
      V p = h.bsdf.p;
      float f0[3] = {invSize * fabsf((p.x - rp) - lo.x), invSize * fabsf((p.y - rp) - lo.y),
                     invSize * fabsf((p.z - rp) - lo.z)};
      float f1[3] = {invSize * fabsf((p.x + rp) - lo.x), invSize * fabsf((p.y + rp) - lo.y),
                     invSize * fabsf((p.z + rp) - lo.z)};
      if (!(std::max(f1[0], std::max(f1[1], f1[2])) < 9.2e18f &&
            std::max(f0[0], std::max(f0[1], f0[2])) < 9.2e18f))
        continue;
      for (long long x = (long long)f0[0]; x <= (long long)f1[0]; x++)
        for (long long y = (long long)f0[1]; y <= (long long)f1[1]; y++)
          for (long long z = (long long)f0[2]; z <= (long long)f1[2]; z++)
            buckets[(size_t)cellBucketOf(x, y, z, cnt)].push_back((int)i);
    }
    // ---- photon pass (tracePhoton/followPhoton, SPPM.hs:170-243)
    uint64_t key = pixelKey(sp->seed, 2 * pass + 1, 0, 0);
    V wlo{INF, INF, INF}, whi{-INF, -INF, -INF};
    for (size_t i = 0; i < S->prims.size(); i++) {
      AabbF b = primBounds(*S, (int)i);
      wlo = V{hmin(wlo.x, b.lo.x), hmin(wlo.y, b.lo.y), hmin(wlo.z, b.lo.z)};
      whi = V{hmax(whi.x, b.hi.x), hmax(whi.y, b.hi.y), hmax(whi.z, b.hi.z)};
    }
    V wc = wlo + (whi - wlo) * V{0.5f, 0.5f, 0.5f};
    float wr = len(whi - wc);
    int T = nthreadsOf(nth);
    if ((int64_t)T > nphot) T = (int)std::max<int64_t>(1, nphot);
    std::vector<std::vector<float>> imgs(T);
    std::vector<std::vector<uint32_t>> ms(T);
    std::vector<uint64_t> ncls(T), nspl(T), nnf(T);
    std::vector<std::thread> th;
    int lc = (int)S->lights.size();
    for (int t = 0; t < T; t++) {
      th.emplace_back([&, t] {
        imgs[t].assign((size_t)width * height * 3, 0.0f);
        ms[t].assign((size_t)st.count, 0u);
        int64_t b = nphot * t / T, e = nphot * (t + 1) / T;
        for (int64_t j = b; j < e; j++) {
          Sampler smp{key, (uint32_t)j, sn, sn, 7, 5};
          float ul = rnd1(smp, 0), uo1, uo2, ud1, ud2;
          rnd2(smp, 0, uo1, uo2);
          rnd2(smp, 1, ud1, ud2);
          int ln = lc == 1 ? 0 : std::min((int)floorf(ul * (float)lc), lc - 1);
          Spec le;
          Ray ray;
          V nl;
          float pdf;
          lightEmit(*S, S->lights[ln], wc, wr, uo1, uo2, ud1, ud2, le, ray, nl, pdf);
          if (lc != 1) pdf = pdf / (float)lc;
          Spec li = sScale(le, absDot(nl, -ray.d) / pdf);
          if (!(pdf > 0 && !isBlack(li))) continue;
          for (int d = 0;; d++) {
            Isect it;
            ncls[t]++;
            if (!sceneIntersect(*S, ray, it)) break;
            V wi = -ray.d;
            const Prim& pr = S->prims[it.prim];
            int mat = pr.is_shape ? S->shapes[pr.index].material : S->meshes[pr.index].material;
            DG dgs = shadingGeometry(*S, pr, it.dg);
            Material mm = hitMaterial(*S, mat, it.dg, dgs);
            Bsdf bsdf = materialBsdf(mm, it.dg, dgs);
            V p = bsdf.p;
            if (bsdfHasNonSpecular(bsdf)) {  // hashLookup (SPPM.hs:307-314)
              float cx = fabsf((p.x - lo.x) * invSize), cy = fabsf((p.y - lo.y) * invSize),
                    cz = fabsf((p.z - lo.z) * invSize);
              if (cx < 9.2e18f && cy < 9.2e18f && cz < 9.2e18f) {
                long long bi = cellBucketOf((long long)cx, (long long)cy, (long long)cz, cnt);
                for (int hi : buckets[(size_t)bi]) {
                  const HitPoint& h = hps[hi];
                  if (!(sqLen(h.bsdf.p - p) <= h.r2)) continue;
                  Spec f = evalBsdf(h.bsdf, h.w, wi);
                  Spec l = sScale(h.F * f * li, 1.0f / (absDot(wi, bsdf.ng) * h.r2 * PI));
                  if (h.px >= 0.0f && h.px < (float)width && h.py >= 0.0f && h.py < (float)height) {
                    if (sNaN(l) || sInf(l)) {
                      nnf[t]++;
                    } else {
                      float x, y, z;
                      spectrumToXYZ(l, x, y, z);
                      float* o = imgs[t].data() + 3 * ((size_t)floorf(h.py) * width + (size_t)floorf(h.px));
                      o[0] = o[0] + x;
                      o[1] = o[1] + y;
                      o[2] = o[2] + z;
                      nspl[t]++;
                    }
                  }
                  int64_t si = st.idx(h.px, h.py);
                  if (si >= 0) ms[t][si]++;
                }
              }
            }
            float ubc = rnd1(smp, 1 + d * 2), u1, u2;
            rnd2(smp, 2 + d, u1, u2);
            BsdfSample bs = sampleBsdf(bsdf, wi, ubc, u1, u2, true);
            float pcont = d > 7 ? 0.8f : 1.0f;
            Spec li2 = sScale(bs.f * li, 1.0f / pcont);
            if (bs.pdf == 0 || isBlack(li2)) break;
            if (rnd1(smp, 2 + d * 2) > pcont) break;
            ray = Ray{p, bs.wi, it.eps, INF};
            li = li2;
          }
        }
      });
    }
    for (auto& x : th) x.join();
    for (int t = 0; t < T; t++) {
      for (size_t k = 0; k < imgs[t].size(); k++) splat_xyz[k] = splat_xyz[k] + imgs[t][k];
      for (int64_t k = 0; k < st.count; k++) m[k] += ms[t][k];
      st_out[0] += ncls[t];
      st_out[2] += nspl[t];
      st_out[3] += nnf[t];
    }
  }
  st_out[1] = (uint64_t)hps.size();
  // ---- statsUpdate (SPPM.hs:272-295)
  float a = sp->alpha;
  for (int64_t i = 0; i < st.count; i++) {
    uint32_t mm = m[i];
    if (mm == 0) continue;
    float n2 = nacc[i] + a * (float)mm;
    float ratio = n2 / (nacc[i] + (float)mm);
    r2[i] = r2[i] * ratio;
    nacc[i] = n2;
    m[i] = 0;
  }
  if (stats) memcpy(stats, st_out, sizeof st_out);
  return BLING_OK;
}

int orc_texture_eval(const orc_scene* s, int node, const float p[3], float u, float v,
                     float out[16]) {
  if (!s || node < 0 || node >= (int)s->tex.size()) return BLING_ERR_INVALID_ARG;
  TexPoint g{V{p[0], p[1], p[2]}, u, v};
  int kind = s->tex[node].kind;
  if (kind >= BLING_TEXN_SCALAR) {
    memset(out, 0, 64);
    out[0] = scalarTex(*s, node, g);
  } else {
    Spec r = spectrumTex(*s, node, g);
    memcpy(out, r.v, 64);
  }
  return BLING_OK;
}
void orc_sunsky_eval(const float east[3], const float sun_dir[3], float turbidity, float u,
                     float v, float out[16]) {
  SkyData sd = initSkyData(mkV(east[0], east[1], east[2]),
                           mkV(sun_dir[0], sun_dir[1], sun_dir[2]), turbidity);
  Spec s = sunSkyEval(sd, u, v);
  memcpy(out, s.v, 64);
}
void orc_rgb_to_spectrum(int illum, float r, float g, float b, float out[16]) {
  Spec s = rgbToSpectrum(illum != 0, r, g, b);
  memcpy(out, s.v, 64);
}
void orc_spectrum_to_xyz(const float s[16], float xyz[3]) {
  Spec sp;
  memcpy(sp.v, s, 64);
  spectrumToXYZ(sp, xyz[0], xyz[1], xyz[2]);
}
void orc_xyz_to_rgb(const float xyz[3], float rgb[3]) {
  xyzToRgb(xyz[0], xyz[1], xyz[2], rgb[0], rgb[1], rgb[2]);
}
float orc_filter_eval(int kind, const float* params, float x, float y) {
  return evalFilter(kind, params, x, y);
}
void orc_filter_table(int kind, const float* params, float out[256]) { filterTable(kind, params, out); }
void orc_random_floats(uint64_t seed, uint64_t pass, int px, int py, uint32_t n, uint32_t dim,
                       int count, float* out) {
  uint64_t k = pixelKey(seed, pass, px, py);
  for (int i = 0; i < count; i++) out[i] = randF(k, n, dim + (uint32_t)i);
}
uint32_t orc_permute(uint32_t i, uint32_t l, uint32_t p) { return permute(i, l, p); }

void orc_xf_translate(float dx, float dy, float dz, float out[32]) {
  setm(out, 1, 0, 0, dx, 0, 1, 0, dy, 0, 0, 1, dz, 0, 0, 0, 1);
  setm(out + 16, 1, 0, 0, -dx, 0, 1, 0, -dy, 0, 0, 1, -dz, 0, 0, 0, 1);
}
void orc_xf_scale(float sx, float sy, float sz, float out[32]) {
  setm(out, sx, 0, 0, 0, 0, sy, 0, 0, 0, 0, sz, 0, 0, 0, 0, 1);
  setm(out + 16, 1.0f / sx, 0, 0, 0, 0, 1.0f / sy, 0, 0, 0, 0, 1.0f / sz, 0, 0, 0, 0, 1);
}
void orc_xf_rotate(int axis, float deg, float out[32]) {
  float s = sinf(radians(deg)), c = cosf(radians(deg));
  if (axis == 0)
    setm(out, 1, 0, 0, 0, 0, c, -s, 0, 0, s, c, 0, 0, 0, 0, 1);
  else if (axis == 1)
    setm(out, c, 0, s, 0, 0, 1, 0, 0, -s, 0, c, 0, 0, 0, 0, 1);
  else
    setm(out, c, -s, 0, 0, s, c, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1);
  for (int i = 0; i < 4; i++)  // transMatrix m
    for (int j = 0; j < 4; j++) out[16 + i * 4 + j] = out[j * 4 + i];
}
void orc_xf_look_at(const float pos[3], const float look[3], const float up[3], float out[32]) {
  V p{pos[0], pos[1], pos[2]}, l{look[0], look[1], look[2]}, u{up[0], up[1], up[2]};
  V dir = normalize(l - p);
  V left = normalize(cross(normalize(u), dir));
  V uu = cross(dir, left);
  setm(out, left.x, uu.x, dir.x, p.x, left.y, uu.y, dir.y, p.y, left.z, uu.z, dir.z, p.z, 0, 0, 0, 1);
  minvert(out, out + 16);
}
void orc_xf_concat(const float a[32], const float b[32], float out[32]) {
  float m[16], i[16];
  mmul(a, b, m);            // mul m1 m2
  mmul(b + 16, a + 16, i);  // mul i2 i1
  memcpy(out, m, 64);
  memcpy(out + 16, i, 64);
}
void orc_xf_perspective(float fov, float n, float f, float out[32]) {
  float iTanAng = 1.0f / tanf(radians(fov) / 2.0f);
  float sc[32];
  orc_xf_scale(iTanAng, iTanAng, 1.0f, sc);
  float pm[32];
  setm(pm, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, f / (f - n), -f * n / (f - n), 0, 0, 1, 0);
  minvert(pm, pm + 16);
  orc_xf_concat(sc, pm, out);
}
void orc_camera_perspective(const float c2w[32], float lr, float fd, float fov, float sx, float sy,
                            bling_camera_desc* out) {
  float p[32];
  orc_xf_perspective(fov, 1e-2f, 1000.0f, p);
  float aspect = sx / sy;
  float s0, s1, s2, s3;
  if (aspect > 1) {
    s0 = -aspect;
    s1 = aspect;
    s2 = -1;
    s3 = 1;
  } else {
    s0 = -1;
    s1 = 1;
    s2 = -1.0f / aspect;
    s3 = 1.0f / aspect;
  }
  float st1[32], st2[32], t[32], tmp[32], s2r[32];
  orc_xf_scale(sx, sy, 1, st1);
  orc_xf_scale(1.0f / (s1 - s0), 1.0f / (s2 - s3), 1, st2);
  orc_xf_translate(-s0, -s3, 0, t);
  orc_xf_concat(st2, st1, tmp);  // t <> (st2 <> st1): <> is infixr
  orc_xf_concat(t, tmp, s2r);
  float r2s[32], pinv[32], r2c[32];
  memcpy(r2s, s2r + 16, 64);
  memcpy(r2s + 16, s2r, 64);
  memcpy(pinv, p + 16, 64);
  memcpy(pinv + 16, p, 64);
  orc_xf_concat(r2s, pinv, r2c);
  memcpy(out->c2w, c2w, 64);
  memcpy(out->c2w_inv, c2w + 16, 64);
  memcpy(out->r2c, r2c, 64);
  memcpy(out->r2c_inv, r2c + 16, 64);
  out->lens_radius = lr;
  out->focal_distance = fd;
  // w2r = w2s <> s2r with w2s = inverse c2w <> p; ap = pw * ph
  float c2wi[32], w2s[32], w2r[32];
  memcpy(c2wi, c2w + 16, 64);
  memcpy(c2wi + 16, c2w, 64);
  orc_xf_concat(c2wi, p, w2s);
  orc_xf_concat(w2s, s2r, w2r);
  memcpy(out->w2r, w2r, 64);
  float fl = tanf(radians(fov) / 2.0f);
  float pw = fl * (s1 - s0) / sx;
  float ph = fl * (s3 - s2) / sy;
  out->pixel_area = pw * ph;
  out->reserved = 0;
}

int orc_light_pass(const orc_scene* S, int32_t width, int32_t height, uint64_t seed, uint64_t pass,
                   int32_t max_depth, int64_t first, int64_t count, float* splat_xyz, int nth,
                   uint64_t stats[4]) {
  if (width <= 0 || height <= 0 || count < 0 || first < 0) return BLING_ERR_INVALID_ARG;
  // worldBounds of the scene's primitives (Primitive/KdTree.hs:111) and its
  // bounding sphere (AABB.hs:53-66)
  V lo{INF, INF, INF}, hi{-INF, -INF, -INF};
  for (size_t i = 0; i < S->prims.size(); i++) {
    AabbF b = primBounds(*S, (int)i);
    lo = V{hmin(lo.x, b.lo.x), hmin(lo.y, b.lo.y), hmin(lo.z, b.lo.z)};
    hi = V{hmax(hi.x, b.hi.x), hmax(hi.y, b.hi.y), hmax(hi.z, b.hi.z)};
  }
  V wc = lo + (hi - lo) * V{0.5f, 0.5f, 0.5f};
  float wr = len(hi - wc);
  int T = nthreadsOf(nth);
  if ((int64_t)T > count) T = (int)std::max<int64_t>(1, count);
  std::vector<std::vector<float>> imgs(T);
  std::vector<Counters> cs(T);
  std::vector<uint64_t> sp(T), nf(T);
  std::vector<std::thread> th;
  for (int t = 0; t < T; t++) {
    th.emplace_back([&, t] {
      imgs[t].assign((size_t)width * height * 3, 0.0f);
      SplatImg img{width, height, imgs[t].data()};
      int64_t b = first + count * t / T, e = first + count * (t + 1) / T;
      for (int64_t g = b; g < e; g++) tracePhoton(*S, seed, pass, (uint64_t)g, wc, wr, max_depth, img, cs[t]);
      sp[t] = img.splats;
      nf[t] = img.nonfinite;
    });
  }
  for (auto& x : th) x.join();
  uint64_t st[4] = {0, 0, 0, 0};
  for (int t = 0; t < T; t++) {
    for (size_t k = 0; k < imgs[t].size(); k++) splat_xyz[k] = splat_xyz[k] + imgs[t][k];
    st[0] += cs[t].closest;
    st[1] += cs[t].any;
    st[2] += sp[t];
    st[3] += nf[t];
  }
  if (stats) memcpy(stats, st, sizeof st);
  return BLING_OK;
}

}  // extern "C"
