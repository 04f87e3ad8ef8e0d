// Photon emission shared by the light tracer (lighttrace.cu) and SPPM
// (sppm.cu): the emitted-ray sample of every light kind.
#pragma once
#include "wavefront.cuh"

namespace bgpu {

// the photon's generator key (photons of a pass are numbered from 0)
__device__ __forceinline__ uint64_t photonKey(uint64_t seed, uint64_t pass, uint64_t photon) {
  return pixelKey(seed, pass, -0x4c54, (int)(uint32_t)(photon >> 32));
}

// sample' (Light.hs:166-213): emitted radiance r, the ray leaving the light,
// the normal there and the pdf
static __device__ void lightEmit(const DevAccel& A, const DevShading& S, const DLight& l, V3 wc, float wr,
                          float uo1, float uo2, float ud1, float ud2, Spec& r, Ray& ray, V3& ns,
                          float& pd) {
  if (l.kind == DLIGHT_AREA) {
    const DShape& s = A.shapes[l.shape];
    V3 orgp, nsp;
    sampleShapeP(s, uo1, uo2, orgp, nsp);  // sampleShape'
    V3 org = transPoint(s.o2w, orgp);
    ns = normalize(transNormal(s.w2o, nsp));
    V3 wi = localToWorld(coordinateSystem(ns), cosineSampleHemisphere(ud1, ud2));
    pd = kInvPi * (1.0f / shapeArea(s)) * absDot(ns, wi);  // shapePdf' = 1 / area
    ray = Ray{org, wi, 1e-3f, INFINITY};
    r = sLoad(S.shape_emission + 16 * l.shape);
    return;
  }
  V3 lv{l.vec[0], l.vec[1], l.vec[2]};
  if (l.kind == DLIGHT_DIRECTIONAL) {
    LC c = coordinateSystem(lv);  // coordinateSystem''
    float d1, d2;
    concentricSampleDisk(uo1, uo2, d1, d2);
    V3 pdisk = wc + sv(wr, sv(d1, c.s) + sv(d2, c.t));
    ns = -lv;
    ray = Ray{pdisk + sv(wr, lv), ns, 0, INFINITY};
    pd = 1.0f / (kPi * wr * wr);
    r = sLoad(l.spec);
    return;
  }
  if (l.kind == DLIGHT_POINT) {
    V3 d = uniformSampleSphere(ud1, ud2);
    ray = Ray{lv, d, 0, INFINITY};
    pd = 1.0f / (2.0f * kPi);  // uniformSpherePdf (Montecarlo.hs:188-190)
    ns = d;
    r = sLoad(l.spec);
    return;
  }
  // infinite: sampleContinuous2D over the map, then a disk across the scene
  float v, pdf1, u, pdf0;
  int im, iu;
  sampleContinuous1D(l.cond_int, l.marg_cdf, l.env_h, l.marg_int, ud2, v, pdf1, im);
  sampleContinuous1D(l.cond_func + (size_t)im * l.env_w, l.cond_cdf + (size_t)im * (l.env_w + 1),
                     l.env_w, __ldg(l.cond_int + im), ud1, u, pdf0, iu);
  float mapPdf = pdf0 * pdf1;
  if (mapPdf == 0) {  // emptySample'
    r = sConst(0);
    ray = Ray{V3{0, 0, 0}, V3{0, 1, 0}, 0, 0};
    ns = V3{0, 1, 0};
    pd = 0;
    return;
  }
  r = envEval(l, u, v);
  float phi = u * 2.0f * kPi, theta = v * kPi;  // cartToSph
  V3 dl{sinf(theta) * cosf(phi), sinf(theta) * sinf(phi), cosf(theta)};
  V3 d = transVector(l.l2w, dl);
  LC c = coordinateSystem(-d);
  float d1, d2;
  concentricSampleDisk(uo1, uo2, d1, d2);
  V3 pDisk = wc + sv(wr, sv(d1, c.s) + sv(d2, c.t));
  ray = Ray{pDisk + sv(wr, d), -d, 0, INFINITY};
  float sint = sinf(theta);
  float pdDir = mapPdf / (2.0f * kPi * kPi * sint);
  float pdArea = 1.0f / (kPi * wr * wr);
  pd = sint == 0 ? 0.0f : pdDir * pdArea;
  ns = d;
}

}  // namespace bgpu
