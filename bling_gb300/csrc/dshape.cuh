// Analytic shapes on the device: ray/shape intersection in object space
// (src/lib/Graphics/Bling/Shape.hs:81-284), placed in the world by mkGeom
// (Primitive/Geometry.hs:14-36).  Same arithmetic order as the reference.
#pragma once
#include "dmath.cuh"

namespace bgpu {

enum { SHAPE_SPHERE = 0, SHAPE_QUAD = 1, SHAPE_BOX = 2, SHAPE_DISK = 3, SHAPE_CYLINDER = 4 };

struct DShape {
  int kind;
  int material;
  int light_id;  // index in the scene light list, -1 when not emissive
  int pad;
  float p[8];
  float o2w[16];
  float w2o[16];
};

// the local differential geometry of a shape hit (DifferentialGeometry.hs:26-36)
struct DGeo {
  V3 p, n, dpdu, dpdv;
  float u, v;
  V3 dndu, dndv;
};

// mkDg (DifferentialGeometry.hs:41-51)
BHD DGeo mkDg(V3 p, float u, float v, V3 dpdu, V3 dpdv, V3 dndu, V3 dndv) {
  return DGeo{p, normalize(cross(dpdu, dpdv)), dpdu, dpdv, u, v, dndu, dndv};
}
// mkDg' (DifferentialGeometry.hs:53-56): u = v = 0, no normal derivatives
BHD DGeo mkDg2(V3 p, V3 n) {
  LC c = coordinateSystem(n);
  return DGeo{p, n, c.s, c.t, 0.0f, 0.0f, V3{0, 0, 0}, V3{0, 0, 0}};
}

// solveQuadric (Math.hs:124-139)
BHD bool solveQuadric(float a, float b, float c, float& t0, float& t1) {
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
BHD bool intersectAABB(V3 bmin, V3 bmax, const Ray& r) {
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
  return !(near > far);
}

// Shape.intersect (object space).  WANT_DG: also build the local DG.
template <bool WANT_DG>
BHD bool shapeIntersect(const DShape& s, const Ray& ray, float& t_out, float& e_out, DGeo* dg) {
  const V3 ro = ray.o, rd = ray.d;
  const float tmin = ray.tmin, tmax = ray.tmax;
  switch (s.kind) {
    case SHAPE_BOX: {
      V3 pmin{s.p[0], s.p[1], s.p[2]}, pmax{s.p[3], s.p[4], s.p[5]};
      float near = -INFINITY, far = INFINITY;
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
      t_out = t;
      e_out = 5e-4f * t;
      if (WANT_DG) {
        V3 p = rayAt(ray, t);
        float half = (comp(pmin, dd) + comp(pmax, dd)) / 2.0f;
        float dir = comp(p, dd) > half ? 1.0f : -1.0f;
        *dg = mkDg2(p, normalize(setComp(dd, dir, v3(0, 0, 0))));
      }
      return true;
    }
    case SHAPE_CYLINDER: {
      float r = s.p[0], zmin = s.p[1], zmax = s.p[2], phimax = s.p[3];
      float a = rd.x * rd.x + rd.y * rd.y;
      float b = 2.0f * (rd.x * ro.x + rd.y * ro.y);
      float c = ro.x * ro.x + ro.y * ro.y - r * r;
      float t0, t1;
      if (!solveQuadric(a, b, c, t0, t1)) return false;
      if (t0 > tmax) return false;
      if (t1 < tmin) return false;
      V3 ph0 = rayAt(ray, t0), ph1 = rayAt(ray, t1);
      float phi0 = atan2p(ph0.y, ph0.x), phi1 = atan2p(ph1.y, ph1.x);
      V3 ph;
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
      t_out = t;
      e_out = 5e-4f * t;
      if (WANT_DG) {
        V3 dpdu{-phimax * ph.y, phimax * ph.x, 0};
        V3 dpdv{0, 0, zmax - zmin};
        *dg = mkDg2(ph, normalize(cross(dpdu, dpdv)));
      }
      return true;
    }
    case SHAPE_DISK: {
      float h = s.p[0], rad = s.p[1], irad = s.p[2], phimax = s.p[3];
      if (fabsf(rd.z) < 1e-7f) return false;
      float t = (h - ro.z) / rd.z;
      if (t < tmin || t > tmax) return false;
      V3 p = rayAt(ray, t);
      float d2 = p.x * p.x + p.y * p.y;
      if (d2 > rad * rad || d2 < irad * irad) return false;
      if (atan2p(p.y, p.x) > phimax) return false;
      t_out = t;
      e_out = 5e-4f * t;
      if (WANT_DG) *dg = mkDg2(p, v3(0, 0, -1));
      return true;
    }
    case SHAPE_QUAD: {
      float sx = s.p[0], sy = s.p[1];
      if (fabsf(rd.z) < 1e-7f) return false;
      float t = -(ro.z) / rd.z;
      if (t < tmin || t > tmax) return false;
      V3 p = rayAt(ray, t);
      if (fabsf(p.x) > sx || fabsf(p.y) > sy) return false;
      t_out = t;
      e_out = 5e-4f * t;
      if (WANT_DG) {  // u, v across the quad (Shape.hs:169-171)
        float u = (sx + p.x) / (2.0f * sx), v = (sy + p.y) / (2.0f * sy);
        *dg = mkDg(p, u, v, v3(sx, 0, 0), v3(0, sy, 0), v3(0, 0, 0), v3(0, 0, 0));
      }
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
      t_out = t;
      e_out = 5e-4f * t;
      if (WANT_DG) {
        V3 p = rayAt(ray, t);
        const float thetaMax = 0.0f, thetaMin = kPi, phiMax = 2.0f * kPi;
        float theta = acosf(hclamp(p.z / r, -1, 1));
        float zradius = sqrtf(p.x * p.x + p.y * p.y);
        float invz = 1.0f / zradius;
        float cosphi = p.x * invz, sinphi = p.y * invz;
        V3 dpdu{-phiMax * p.y, phiMax * p.x, 0};
        float k = thetaMax - thetaMin;
        V3 dpdv = V3{p.z * cosphi, p.z * sinphi, -r * sinf(theta)} * V3{k, k, k};
        float u = atan2p(p.y, p.x) / phiMax, v = (theta - thetaMin) / k;
        // the normal's derivatives from the fundamental forms (Shape.hs:209-229)
        V3 d2Pduu = V3{-phiMax * phiMax, -phiMax * phiMax, -phiMax * phiMax} * V3{p.x, p.y, 0};
        float cuv = k * p.z * phiMax;
        V3 d2Pduv = V3{cuv, cuv, cuv} * V3{-sinphi, cosphi, 0};
        float cvv = -k * k;
        V3 d2Pdvv = V3{cvv, cvv, cvv} * V3{p.x, p.y, p.z};
        float E1 = dot(dpdu, dpdu), F1 = dot(dpdu, dpdv), G1 = dot(dpdv, dpdv);
        V3 n1 = normalize(cross(dpdu, dpdv));
        float e = dot(n1, d2Pduu), f = dot(n1, d2Pduv), g = dot(n1, d2Pdvv);
        float invEGF2 = 1.0f / (E1 * G1 - F1 * F1);
        float a = (f * F1 - e * G1) * invEGF2, b = (e * F1 - f * E1) * invEGF2;
        float c = (g * F1 - f * G1) * invEGF2, d = (f * F1 - g * E1) * invEGF2;
        V3 dndu = V3{a, a, a} * dpdu + V3{b, b, b} * dpdv;
        V3 dndv = V3{c, c, c} * dpdu + V3{d, d, d} * dpdv;
        *dg = mkDg(p, u, v, dpdu, dpdv, dndu, dndv);
      }
      return true;
    }
  }
}

// Shape.intersects (object space, Shape.hs:231-284)
BHD bool shapeIntersects(const DShape& s, const Ray& ray) {
  const V3 ro = ray.o, rd = ray.d;
  const float tmin = ray.tmin, tmax = ray.tmax;
  switch (s.kind) {
    case SHAPE_BOX:
      return intersectAABB(V3{s.p[0], s.p[1], s.p[2]}, V3{s.p[3], s.p[4], s.p[5]}, ray);
    case SHAPE_CYLINDER: {
      float r = s.p[0], zmin = s.p[1], zmax = s.p[2], phimax = s.p[3];
      float a = rd.x * rd.x + rd.y * rd.y;
      float b = 2.0f * (rd.x * ro.x + rd.y * ro.y);
      float c = ro.x * ro.x + ro.y * ro.y - r * r;
      float t0, t1;
      if (!solveQuadric(a, b, c, t0, t1)) return false;
      if (t0 > tmax) return false;
      if (t1 < tmin) return false;
      V3 ph0 = rayAt(ray, t0), ph1 = rayAt(ray, t1);
      float phi0 = atan2p(ph0.y, ph0.x), phi1 = atan2p(ph1.y, ph1.x);
      if (t0 > tmin && ph0.z > zmin && ph0.z < zmax && phi0 <= phimax) return true;
      return t1 < tmax && ph1.z > zmin && ph1.z < zmax && phi1 <= phimax && t1 <= tmax;
    }
    case SHAPE_DISK: {
      float h = s.p[0], rad = s.p[1], irad = s.p[2], phimax = s.p[3];
      if (fabsf(rd.z) < 1e-7f) return false;
      float t = (h - ro.z) / rd.z;
      if (t < tmin || t > tmax) return false;
      V3 p = rayAt(ray, t);
      float d2 = p.x * p.x + p.y * p.y;
      if (d2 > rad * rad || d2 < irad * irad) return false;
      return !(atan2p(p.y, p.x) > phimax);
    }
    case SHAPE_QUAD: {
      if (fabsf(rd.z) < 1e-7f) return false;
      float t = -(ro.z) / rd.z;
      if (t < tmin || t > tmax) return false;
      V3 p = rayAt(ray, t);
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

// area (Shape.hs:314-328)
BHD float shapeArea(const DShape& s) {
  switch (s.kind) {
    case SHAPE_BOX: {
      float h = s.p[3] - s.p[0], w = s.p[4] - s.p[1], l = s.p[5] - s.p[2];
      return 2.0f * (h * w + h * l + w * l);
    }
    case SHAPE_CYLINDER: return 2.0f * kPi * s.p[0] * (s.p[2] - s.p[1]);
    case SHAPE_DISK: {
      float rmin2 = s.p[2] * s.p[2], rmax2 = s.p[1] * s.p[1];
      return kPi * (rmax2 - rmin2);
    }
    case SHAPE_QUAD: return 4.0f * s.p[0] * s.p[1];
    default: return s.p[0] * s.p[0] * 4.0f * kPi;
  }
}

}  // namespace bgpu
