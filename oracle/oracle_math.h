// Oracle math: binary32 restatement of bling's vector, ray and transform
// arithmetic.  TEST INFRASTRUCTURE ONLY -- this is the parity checker for the
// GPU path; nothing in the product links it.
//
// Every expression keeps the reference's operation order and is compiled with
// -ffp-contract=off, so each + - * / rounds once as GHC's Float arithmetic does.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace orc {

// GHC's default Ord methods: min x y = if x <= y then x else y (Math.hs users)
static inline float hmin(float a, float b) { return a <= b ? a : b; }
static inline float hmax(float a, float b) { return a <= b ? b : a; }
// clamp (Math.hs:78-87)
static inline float clampf(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }

static const float PI = 3.14159265358979323846f;
static const float TWO_PI = 2.0f * PI;          // twoPi = 2.0 * pi (Math.hs:57-59)
static const float INV_PI = 1.0f / PI;          // invPi (Math.hs:49-51)
static const float INV_TWO_PI = 1.0f / (2.0f * PI);  // invTwoPi (Math.hs:53-55)
static const float INF = INFINITY;

// radians x = x / 180 * pi (Math.hs:62-66)
static inline float radians(float x) { return x / 180.0f * PI; }

// GHC.Float's RealFloat default atan2, which Float uses (built on atanf).
static inline float hatan2(float y, float x) {
  if (x > 0) return atanf(y / x);
  if (x == 0 && y > 0) return PI / 2;
  if (x < 0 && y > 0) return PI + atanf(y / x);
  bool ny = std::signbit(y) && y == 0, nx = std::signbit(x) && x == 0;
  if ((x <= 0 && y < 0) || (x < 0 && ny) || (nx && ny)) return -hatan2(-y, x);
  if (y == 0 && (x < 0 || nx)) return PI;
  if (x == 0 && y == 0) return y;
  return x + y;
}
// atan2' (Math.hs:69-75)
static inline float atan2p(float y, float x) {
  float a = hatan2(y, x);
  return a < 0 ? a + TWO_PI : a;
}
// lerp t v1 v2 = (1 - t) * v1 + t * v2 (Math.hs:108-110)
static inline float lerp(float t, float a, float b) { return (1.0f - t) * a + t * b; }

struct V {
  float x, y, z;
};
static inline V mkV(float x, float y, float z) { return V{x, y, z}; }
static inline V operator+(V a, V b) { return V{a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V operator-(V a, V b) { return V{a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V operator*(V a, V b) { return V{a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline V operator-(V a) { return V{-a.x, -a.y, -a.z}; }
// f *# v = vpromote f * v (Math.hs:207-209)
static inline V sv(float f, V v) { return V{f * v.x, f * v.y, f * v.z}; }
// Math.hs:328-353
static inline float sqLen(V v) { return v.x * v.x + v.y * v.y + v.z * v.z; }
static inline float len(V v) { return sqrtf(sqLen(v)); }
static inline V cross(V u, V v) {
  return V{u.y * v.z - u.z * v.y, -(u.x * v.z - u.z * v.x), u.x * v.y - u.y * v.x};
}
static inline float dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float absDot(V a, V b) { return fabsf(dot(a, b)); }
static inline V normalize(V v) {
  if (sqLen(v) != 0) {
    float il = 1.0f / len(v);
    return V{v.x * il, v.y * il, v.z * il};
  }
  return V{0, 1, 0};
}
static inline float comp(V v, int d) { return d == 0 ? v.x : (d == 1 ? v.y : v.z); }
static inline V setComp(int d, float t, V v) {
  if (d == 0) return V{t, v.y, v.z};
  if (d == 1) return V{v.x, t, v.z};
  return V{v.x, v.y, t};
}
static inline bool isZeroV(V v) { return v.x == 0 && v.y == 0 && v.z == 0; }

struct Ray {
  V o, d;
  float tmin, tmax;
};
// rayAt (Math.hs:388-390)
static inline V rayAt(const Ray& r, float t) { return r.o + V{r.d.x * t, r.d.y * t, r.d.z * t}; }

// LocalCoordinates / coordinateSystem (Math.hs:408-449)
struct LC {
  V s, t, n;
};
static inline LC coordinateSystem(V v) {
  if (fabsf(v.x) > fabsf(v.y)) {
    float il = 1.0f / sqrtf(v.x * v.x + v.z * v.z);
    V v2{-v.z * il, 0, v.x * il};
    return LC{v2, cross(v, v2), v};
  }
  float il = 1.0f / sqrtf(v.y * v.y + v.z * v.z);
  V v2{0, v.z * il, -v.y * il};
  return LC{v2, cross(v, v2), v};
}
static inline V worldToLocal(const LC& c, V v) { return V{dot(v, c.s), dot(v, c.t), dot(v, c.n)}; }
static inline V localToWorld(const LC& c, V v) {
  return V{c.s.x * v.x + c.t.x * v.y + c.n.x * v.z, c.s.y * v.x + c.t.y * v.y + c.n.y * v.z,
           c.s.z * v.x + c.t.z * v.y + c.n.z * v.z};
}

// Transform = (matrix, inverted), row-major 4x4 (Transform.hs:124-127)
struct Xf {
  float m[16];
  float i[16];
};
static inline Xf xfInverse(const Xf& t) {
  Xf r;
  memcpy(r.m, t.i, sizeof r.m);
  memcpy(r.i, t.m, sizeof r.i);
  return r;
}
// transPoint (Transform.hs:247-256)
static inline V transPoint(const float* m, V p) {
  float xp = m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3];
  float yp = m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7];
  float zp = m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11];
  float wp = m[12] * p.x + m[13] * p.y + m[14] * p.z + m[15];
  if (wp == 1) return V{xp, yp, zp};
  return V{xp / wp, yp / wp, zp / wp};
}
// transVector (Transform.hs:259-264)
static inline V transVector(const float* m, V v) {
  return V{m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
           m[8] * v.x + m[9] * v.y + m[10] * v.z};
}
// transNormal uses the inverted matrix, transposed (Transform.hs:267-272)
static inline V transNormal(const float* mi, V n) {
  return V{mi[0] * n.x + mi[4] * n.y + mi[8] * n.z, mi[1] * n.x + mi[5] * n.y + mi[9] * n.z,
           mi[2] * n.x + mi[6] * n.y + mi[10] * n.z};
}
// transRay (Transform.hs:275-278)
static inline Ray transRay(const float* m, const Ray& r) {
  return Ray{transPoint(m, r.o), transVector(m, r.d), r.tmin, r.tmax};
}

}  // namespace orc
