// Device math for the path-tracing core: the reference's vector, ray and
// transform arithmetic (src/lib/Graphics/Bling/Math.hs, Transform.hs) in IEEE
// binary32 with the reference's operation order.  This translation unit is
// compiled with -fmad=false, so no multiply-add is contracted and every
// + - * / rounds once, as GHC's Float arithmetic does; intersection results
// (hit distance, primitive) are therefore bit-identical to the reference's.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#define BHD __host__ __device__ __forceinline__

namespace bgpu {

static constexpr float kPi = 3.14159265358979323846f;

// GHC's default Ord methods (min x y = if x <= y then x else y)
BHD float hmin(float a, float b) { return a <= b ? a : b; }
BHD float hmax(float a, float b) { return a <= b ? b : a; }
BHD float hclamp(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }

struct V3 {
  float x, y, z;
};
BHD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
BHD V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
BHD V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
BHD V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
BHD V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
// f *# v (Math.hs:207-209)
BHD V3 sv(float f, V3 v) { return V3{f * v.x, f * v.y, f * v.z}; }
// Math.hs:328-353
BHD float sqLen(V3 v) { return v.x * v.x + v.y * v.y + v.z * v.z; }
BHD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
BHD float absDot(V3 a, V3 b) { return fabsf(dot(a, b)); }
BHD V3 cross(V3 u, V3 v) {
  return V3{u.y * v.z - u.z * v.y, -(u.x * v.z - u.z * v.x), u.x * v.y - u.y * v.x};
}
BHD V3 normalize(V3 v) {
  float s = sqLen(v);
  if (s != 0) {
    float il = 1.0f / sqrtf(s);
    return V3{v.x * il, v.y * il, v.z * il};
  }
  return V3{0, 1, 0};
}
BHD float comp(V3 v, int d) { return d == 0 ? v.x : (d == 1 ? v.y : v.z); }
BHD V3 setComp(int d, float t, V3 v) {
  return d == 0 ? V3{t, v.y, v.z} : (d == 1 ? V3{v.x, t, v.z} : V3{v.x, v.y, t});
}

struct Ray {
  V3 o, d;
  float tmin, tmax;
};
// rayAt (Math.hs:388-390)
BHD V3 rayAt(const Ray& r, float t) { return r.o + V3{r.d.x * t, r.d.y * t, r.d.z * t}; }

// transPoint / transVector / transNormal (Transform.hs:247-272)
BHD V3 transPoint(const float* m, V3 p) {
  float xp = m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3];
  float yp = m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7];
  float zp = m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11];
  float wp = m[12] * p.x + m[13] * p.y + m[14] * p.z + m[15];
  if (wp == 1) return V3{xp, yp, zp};
  return V3{xp / wp, yp / wp, zp / wp};
}
BHD V3 transVector(const float* m, V3 v) {
  return V3{m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
            m[8] * v.x + m[9] * v.y + m[10] * v.z};
}
BHD V3 transNormal(const float* mi, V3 n) {
  return V3{mi[0] * n.x + mi[4] * n.y + mi[8] * n.z, mi[1] * n.x + mi[5] * n.y + mi[9] * n.z,
            mi[2] * n.x + mi[6] * n.y + mi[10] * n.z};
}
BHD Ray transRay(const float* m, const Ray& r) {
  return Ray{transPoint(m, r.o), transVector(m, r.d), r.tmin, r.tmax};
}

// coordinateSystem (Math.hs:413-425)
struct LC {
  V3 s, t, n;
};
BHD LC coordinateSystem(V3 v) {
  if (fabsf(v.x) > fabsf(v.y)) {
    float il = 1.0f / sqrtf(v.x * v.x + v.z * v.z);
    V3 v2{-v.z * il, 0, v.x * il};
    return LC{v2, cross(v, v2), v};
  }
  float il = 1.0f / sqrtf(v.y * v.y + v.z * v.z);
  V3 v2{0, v.z * il, -v.y * il};
  return LC{v2, cross(v, v2), v};
}
BHD V3 worldToLocal(const LC& c, V3 v) { return V3{dot(v, c.s), dot(v, c.t), dot(v, c.n)}; }
BHD V3 localToWorld(const LC& c, V3 v) {
  return V3{c.s.x * v.x + c.t.x * v.y + c.n.x * v.z, c.s.y * v.x + c.t.y * v.y + c.n.y * v.z,
            c.s.z * v.x + c.t.z * v.y + c.n.z * v.z};
}

// GHC.Float's default atan2 for Float (built on atanf)
BHD float hatan2(float y, float x) {
  for (int flip = 0; flip < 2; flip++) {
    if (x > 0) return flip ? -atanf(y / x) : atanf(y / x);
    if (x == 0 && y > 0) return flip ? -(kPi / 2) : kPi / 2;
    if (x < 0 && y > 0) return flip ? -(kPi + atanf(y / x)) : kPi + atanf(y / x);
    bool ny = signbit(y) && y == 0, nx = signbit(x) && x == 0;
    if ((x <= 0 && y < 0) || (x < 0 && ny) || (nx && ny)) {
      if (flip) break;  // cannot recurse twice: -y is non-negative
      y = -y;
      continue;
    }
    if (y == 0 && (x < 0 || nx)) return flip ? -kPi : kPi;
    if (x == 0 && y == 0) return flip ? -y : y;
    return flip ? -(x + y) : x + y;
  }
  return x + y;
}
// atan2' (Math.hs:69-75)
BHD float atan2p(float y, float x) {
  float a = hatan2(y, x);
  return a < 0 ? a + 2.0f * kPi : a;
}
BHD float hlerp(float t, float a, float b) { return (1.0f - t) * a + t * b; }

}  // namespace bgpu
