// Texture expressions on the device (src/lib/Graphics/Bling/Texture.hs) and
// bump mapping (Reflection.hs:344-377).  A material parameter that names a
// texture node is evaluated per hit at the shading geometry: the shading
// point p (world space) and the surface parameters (u, v).  Nodes form
// trees (children before parents, depth checked at upload), evaluated in the
// reference's operation order by functions unrolled over the depth, so no
// call is recursive and the stack each kernel needs is known; images and
// gradients are read from device arrays the scene upload prepares.
#pragma once
#include "dmath.cuh"
#include "integrator.h"
#include "spectrum_tables.h"

namespace bgpu {

// the part of the shading DifferentialGeometry textures read
struct TexGeo {
  V3 p;
  float u, v;
};

static __device__ const uint8_t kNoisePerm[256] = {BLING_NOISE_PERM_LIST};

// noisePerms ! i for i < 512 (the list is the permutation twice)
__device__ __forceinline__ int noisePerm(int i) { return (int)__ldg(kNoisePerm + (i & 255)); }

// grad (Texture.hs:384-393)
__device__ __forceinline__ float noiseGrad(int x, int y, int z, float dx, float dy, float dz) {
  int h = noisePerm(noisePerm(noisePerm(x) + y) + z) & 15;
  float u = (h < 8 || h == 12 || h == 13) ? dx : dy;
  float v = (h < 4 || h == 12 || h == 13) ? dy : dz;
  return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
}
// noiseWeight (Texture.hs:378-382)
__device__ __forceinline__ float noiseWeight(float t) {
  float t3 = t * t * t;
  float t4 = t3 * t;
  return 6.0f * t4 * t - 15.0f * t4 + 10.0f * t3;
}
// floor :: Float -> Int
__device__ __forceinline__ long long floorInt(float x) { return (long long)floorf(x); }

// perlin3d (Texture.hs:348-376)
static __device__ float perlin3d(float x, float y, float z) {
  long long fx = floorInt(x), fy = floorInt(y), fz = floorInt(z);
  float dx = x - (float)fx, dy = y - (float)fy, dz = z - (float)fz;
  int ix = (int)(fx & 255), iy = (int)(fy & 255), iz = (int)(fz & 255);
  float w000 = noiseGrad(ix, iy, iz, dx, dy, dz);
  float w100 = noiseGrad(ix + 1, iy, iz, dx - 1.0f, dy, dz);
  float w010 = noiseGrad(ix, iy + 1, iz, dx, dy - 1.0f, dz);
  float w110 = noiseGrad(ix + 1, iy + 1, iz, dx - 1.0f, dy - 1.0f, dz);
  float w001 = noiseGrad(ix, iy, iz + 1, dx, dy, dz - 1.0f);
  float w101 = noiseGrad(ix + 1, iy, iz + 1, dx - 1.0f, dy, dz - 1.0f);
  float w011 = noiseGrad(ix, iy + 1, iz + 1, dx, dy - 1.0f, dz - 1.0f);
  float w111 = noiseGrad(ix + 1, iy + 1, iz + 1, dx - 1.0f, dy - 1.0f, dz - 1.0f);
  float wx = noiseWeight(dx), wy = noiseWeight(dy), wz = noiseWeight(dz);
  float x00 = hlerp(wx, w000, w100), x10 = hlerp(wx, w010, w110);
  float x01 = hlerp(wx, w001, w101), x11 = hlerp(wx, w011, w111);
  float y0 = hlerp(wy, x00, x10), y1 = hlerp(wy, x01, x11);
  return hlerp(wz, y0, y1);
}

// fbm octaves omega (Texture.hs:328-337): the octaves' terms summed from 0
// left to right, lambda_k = 1.99^k and o_k = omega^k by repeated products
static __device__ float fbm(int octaves, float omega, V3 p) {
  float acc = 0.0f, l = 1.0f, o = 1.0f;
  for (int k = 0; k < octaves; k++) {
    acc = acc + o * perlin3d(p.x * l, p.y * l, p.z * l);
    l = 1.99f * l;
    o = omega * o;
  }
  return acc;
}

// cellNoise (Texture.hs:250-300): Worley noise with 1..9 points per cell
__device__ __forceinline__ long long cellLcg(long long x) {
  return (1103515245LL * x + 12345LL) % 4294967296LL;
}
__device__ __forceinline__ int cellPoints(long long value) {  // prob
  if (value < 393325350LL) return 1;
  if (value < 1022645910LL) return 2;
  if (value < 1861739990LL) return 3;
  if (value < 2700834071LL) return 4;
  if (value < 3372109335LL) return 5;
  if (value < 3819626178LL) return 6;
  if (value < 4075350088LL) return 7;
  if (value < 4203212043LL) return 8;
  return 9;
}
static __device__ float cellNoise(int dist, V3 p) {
  long long ox = floorInt(p.x), oy = floorInt(p.y), oz = floorInt(p.z);
  float best = 0.0f;
  bool first = true;
  for (int cx = -1; cx <= 1; cx++)
    for (int cy = -1; cy <= 1; cy++)
      for (int cz = -1; cz <= 1; cz++) {
        long long X = cx + ox, Y = cy + oy, Z = cz + oz;
        long long h = (X * 73856093LL) ^ (Y * 19349663LL) ^ (Z * 83492791LL);
        h = (h < 0 ? -h : h) % 4294967296LL;
        long long u = cellLcg(h);
        int n = cellPoints(u);
        for (int k = 0; k < n; k++) {
          long long u1 = cellLcg(u), u2 = cellLcg(u1), u3 = cellLcg(u2);
          V3 q{(float)X + (float)u1 / 4294967296.0f, (float)Y + (float)u2 / 4294967296.0f,
               (float)Z + (float)u3 / 4294967296.0f};
          u = u3;
          V3 d = p - q;
          float e;
          if (dist == 1) {  // sqEuclidianDist
            e = sqLen(d);
          } else if (dist == 2) {  // manhattanDist
            e = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
          } else if (dist == 3) {  // chebyshevDist: maximum of the three
            e = hmax(hmax(fabsf(d.x), fabsf(d.y)), fabsf(d.z));
          } else {  // euclidianDist
            e = sqrtf(sqLen(d));
          }
          best = first ? e : hmin(best, e);
          first = false;
        }
      }
  return best;
}

// quasiCrystal (Texture.hs:302-326): waves at the angles 0, pi/n, ... of
// enumFromThen (each next angle m + m - n of the previous two), summed from
// 0, folded into [0, 1] by wrap
static __device__ float quasiCrystal(int n, float x, float y) {
  const float step = kPi / (float)n;
  float a0 = 0.0f, a1 = step, acc = 0.0f;
  for (int k = 0; k < n; k++) {
    float th = a0;
    float cth = cosf(th), sth = sinf(th);
    acc = acc + (cosf(cth * x + sth * y) + 1.0f) / 2.0f;
    float a2 = a1 + a1 - a0;
    a0 = a1;
    a1 = a2;
  }
  // wrap: properFraction, a negative fraction moved up by one
  long long k = (long long)truncf(acc);
  float v = acc - (float)k;
  if (v < 0) {
    k = k - 1;
    v = 1.0f + v;
  }
  return (k & 1) ? 1.0f - v : v;
}

// a node's 2D mapping (uvMapping, planarMapping, Texture.hs:160-176)
__device__ __forceinline__ void texMap2d(const DTex& t, const TexGeo& g, float& s, float& r) {
  const float* m = t.map;
  if (t.map_kind == 1) {
    s = dot(g.p, V3{m[0], m[1], m[2]}) + m[6];
    r = dot(g.p, V3{m[3], m[4], m[5]}) + m[7];
  } else {
    s = m[0] * g.u + m[2];
    r = m[1] * g.v + m[3];
  }
}
// identityMapping3d w2t (Texture.hs:150-154)
__device__ __forceinline__ V3 texMap3d(const DTex& t, const TexGeo& g) {
  return transPoint(t.map, g.p);
}
// getPixel's texel (Texture.hs:95-101): u and -v scaled to the image,
// floored, wrapped into it
__device__ __forceinline__ size_t texel(const DTex& t, float s, float r) {
  long long px = floorInt(s * (float)t.width) % t.width;
  long long py = floorInt((-r) * (float)t.height) % t.height;
  if (px < 0) px += t.width;
  if (py < 0) py += t.height;
  return (size_t)py * t.width + (size_t)px;
}

// The evaluators are templates over the depth left (D): a node at depth D
// evaluates its children at D - 1, so the call graph has no cycle and the
// kernels' stack size is known at compile time.  Trees are at most
// BLING_TEX_MAX_DEPTH deep (checked at upload), so D = 0 is never reached.
template <int D>
__device__ __noinline__ float texScalarD(const DTex* __restrict__ T, int i, const TexGeo& g);
template <int D>
__device__ __noinline__ void texSpectrumD(const DTex* __restrict__ T, int i, const TexGeo& g,
                                          float* out);
template <>
__device__ __forceinline__ float texScalarD<0>(const DTex* __restrict__, int, const TexGeo&) {
  return 0.0f;
}
template <>
__device__ __forceinline__ void texSpectrumD<0>(const DTex* __restrict__, int, const TexGeo&,
                                                float* out) {
  for (int k = 0; k < 16; k++) out[k] = 0.0f;
}

// a scalar-valued node at g
template <int D>
__device__ __noinline__ float texScalarD(const DTex* __restrict__ T, int i, const TexGeo& g) {
  const DTex& t = T[i];
  switch (t.kind) {
    case 17:  // scaleTexture a s tex
      return t.p[0] + t.p[1] * texScalarD<D - 1>(T, t.a, g);
    case 18: {  // noiseTexture
      V3 q = texMap3d(t, g);
      return perlin3d(q.x, q.y, q.z);
    }
    case 19:  // fbm over the 3D mapping
      return fbm(t.ivalue, t.p[0], texMap3d(t, g));
    case 20:
      return cellNoise(t.ivalue, texMap3d(t, g));
    case 21: {
      float s, r;
      texMap2d(t, g, s, r);
      return quasiCrystal(t.ivalue, s, r);
    }
    case 22: {  // a grey image
      float s, r;
      texMap2d(t, g, s, r);
      return __ldg(t.data + texel(t, s, r));
    }
    default:  // constant
      return t.p[0];
  }
}

// a spectrum-valued node at g, into out
template <int D>
__device__ __noinline__ void texSpectrumD(const DTex* __restrict__ T, int i, const TexGeo& g,
                                          float* out) {
  const DTex& t = T[i];
  switch (t.kind) {
    case 1: {  // spectrumBlend t1 t2 f
      float x = texScalarD<D - 1>(T, t.c, g);
      if (x <= 0) {
        texSpectrumD<D - 1>(T, t.a, g, out);
      } else if (x >= 1) {
        texSpectrumD<D - 1>(T, t.b, g, out);
      } else {
        float v1[16], v2[16];
        texSpectrumD<D - 1>(T, t.a, g, v1);
        texSpectrumD<D - 1>(T, t.b, g, v2);
        for (int k = 0; k < 16; k++) out[k] = v1[k] * (1.0f - x) + v2[k] * x;
      }
      return;
    }
    case 2: {  // checkerBoard: floor (x sx) + floor (y sy) + floor (z sz), even -> t1
      long long c = floorInt(g.p.x * t.p[0]) + floorInt(g.p.y * t.p[1]) + floorInt(g.p.z * t.p[2]);
      texSpectrumD<D - 1>(T, (c & 1) == 0 ? t.a : t.b, g, out);
      return;
    }
    case 3: {  // graphPaper lw m paper lines
      float x, z;
      texMap2d(t, g, x, z);
      float xf = fabsf(x - truncf(x)), zf = fabsf(z - truncf(z));  // properFraction
      float lo = t.p[0] / 2.0f, hi = 1.0f - lo;
      texSpectrumD<D - 1>(T, (xf < lo || zf < lo || xf > hi || zf > hi) ? t.b : t.a, g, out);
      return;
    }
    case 4: {  // gradient
      float f = texScalarD<D - 1>(T, t.c, g);
      const float* st = t.data;
      int n = t.ivalue;
      float pmin = st[0], pmax = st[17 * (n - 1)];
      if (f <= pmin) {
        for (int k = 0; k < 16; k++) out[k] = __ldg(st + 1 + k);
        return;
      }
      if (f >= pmax) {
        for (int k = 0; k < 16; k++) out[k] = __ldg(st + 17 * (n - 1) + 1 + k);
        return;
      }
      int idx = 1;
      while (idx < n - 1 && !(__ldg(st + 17 * idx) > f)) idx++;  // findIndex ((> f) . fst)
      const float* e0 = st + 17 * (idx - 1);
      const float* e1 = st + 17 * idx;
      float w = (f - __ldg(e0)) / (__ldg(e1) - __ldg(e0));
      for (int k = 0; k < 16; k++) out[k] = __ldg(e0 + 1 + k) * (1.0f - w) + __ldg(e1 + 1 + k) * w;
      return;
    }
    case 5: {  // an RGB image
      float s, r;
      texMap2d(t, g, s, r);
      const float* px = t.data + 16 * texel(t, s, r);
      for (int k = 0; k < 16; k++) out[k] = __ldg(px + k);
      return;
    }
    default:  // constant
      for (int k = 0; k < 16; k++) out[k] = t.spectrum[k];
      return;
  }
}

// the evaluators for a tree's root
__device__ __forceinline__ float texScalar(const DTex* __restrict__ T, int i, const TexGeo& g) {
  return texScalarD<BLING_TEX_MAX_DEPTH>(T, i, g);
}
__device__ __forceinline__ void texSpectrum(const DTex* __restrict__ T, int i, const TexGeo& g,
                                            float* out) {
  texSpectrumD<BLING_TEX_MAX_DEPTH>(T, i, g, out);
}

}  // namespace bgpu
