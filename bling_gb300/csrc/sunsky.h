// The reference's sun and sky (SunSky.hs): Perez's sky luminance and
// chromaticity model plus a solar disc, as the lat-long map of an infinite
// light.  The map is evaluated at continuous (u, v) wherever the light needs
// it (le and sample, Light.hs:98-106, 130-141); only the importance
// distribution uses its 640 x 480 raster (mkInfiniteAreaLight's mkDist2D,
// Light.hs:72-82).  skyEval runs on host and device alike; skyInit computes
// the per-light constants (initSky and sunSpectrum', SunSky.hs:45-65, 96-125)
// on the host.  Arithmetic is binary32 in the reference's operation order.
#pragma once
#include <math.h>
#include <string.h>

#include "spectrum_tables.h"

namespace bgpu {

struct SkyModel {
  float sky_sun[3];   // SkyData's sunDir: normalize (worldToLocal basis (normalize sunDir))
  float sun_disc[3];  // the disc's direction: normalize (worldToLocal basis sunDir)
  float sun_theta;    // acos (clamp sunDir.z)
  float px[5], py[5], pY[5];  // Perez coefficients of x, y and Y
  float zx, zy, zY;           // zenith chromaticity and luminance
  float stm;                  // sunThetaMax2
  float s012[9];              // X, Y, Z of the CIE daylight components S0, S1, S2
  float sun_r[16];            // the solar spectrum at the ground (zero below the horizon)
  float illum[7 * 16];        // the illuminant RGB basis (white cyan magenta yellow red green blue)
};

constexpr int kSkyMapW = 640, kSkyMapH = 480;  // mkSunSkyLight's map size

// clamp (Math.hs:78-87): NaN passes through
static inline BLING_HD float skyClamp(float v, float lo, float hi) {
  if (v < lo) return lo;
  if (v > hi) return hi;
  return v;
}

// perez (SunSky.hs:81-86)
static inline BLING_HD float skyPerez(const float p[5], float sunT, float t, float g, float lvz) {
  float csg = cosf(g), cst = cosf(sunT);
  float num = (1.0f + p[0] * expf(p[1] / cosf(t))) * (1.0f + p[2] * expf(p[3] * g)) + p[4] * csg * csg;
  float den = (1.0f + p[0] * expf(p[1])) * (1.0f + p[2] * expf(p[3] * sunT)) + p[4] * cst * cst;
  return lvz * num / den;
}

// the map at (u, v): skySpectrum + sunSpectrum of the direction
// sphToDir (cartToSph (u, v)) (SunSky.hs:17-20, 67-94; Types.hs:31-33;
// Math.hs:141-148)
static inline BLING_HD void skyEval(const SkyModel& m, float u, float v, float out[16]) {
  const float kPiF = 3.14159274101257324f;
  float phi = u * 2.0f * kPiF, theta = v * kPiF;
  float st = sinf(theta);
  float d[3] = {st * cosf(phi), st * sinf(phi), cosf(theta)};
  for (int i = 0; i < 16; i++) out[i] = 0.0f;
  // sky (skySpectrum): black below the horizon of the map's -z axis
  float dz = -d[2];
  if (!(dz < 1e-4f)) {
    float th = acosf(dz);
    float cg = d[0] * m.sky_sun[0] + d[1] * m.sky_sun[1] + d[2] * m.sky_sun[2];
    float g = acosf(skyClamp(cg, -1.0f, 1.0f));
    float x = skyPerez(m.px, m.sun_theta, th, g, m.zx);
    float y = skyPerez(m.py, m.sun_theta, th, g, m.zy);
    float Y = skyPerez(m.pY, m.sun_theta, th, g, m.zY) * 1e-4f;
    // chromaticityToXYZ (Spectrum.hs:221-251)
    float den = 0.0241f + 0.2562f * x - 0.7341f * y;
    float m1 = (-1.3515f - 1.7703f * x + 5.9114f * y) / den;
    float m2 = (0.03f - 31.4424f * x + 30.0717f * y) / den;
    float cx = m.s012[0] + m1 * m.s012[3] + m2 * m.s012[6];
    float cy = m.s012[1] + m1 * m.s012[4] + m2 * m.s012[7];
    float cz = m.s012[2] + m1 * m.s012[5] + m2 * m.s012[8];
    float X = cx * Y / cy, Z = cz * Y / cy;
    // xyzToSpectrum = rgbToSpectrumIllum . xyzToRgb (Spectrum.hs:120-168, 357-358)
    float r = 3.240479f * X - 1.537150f * Y - 0.498535f * Z;
    float gg = (-0.969256f) * X + 1.875991f * Y + 0.041556f * Z;
    float b = 0.055648f * X - 0.204043f * Y + 1.057311f * Z;
    const float* W = m.illum;
    const float* C = m.illum + 16;
    const float* M = m.illum + 32;
    const float* Yb = m.illum + 48;
    const float* R = m.illum + 64;
    const float* G = m.illum + 80;
    const float* B = m.illum + 96;
    for (int i = 0; i < 16; i++) {
      float s;
      if (r <= gg && r <= b)
        s = W[i] * r + (gg <= b ? C[i] * (gg - r) + B[i] * (b - gg) : C[i] * (b - r) + G[i] * (gg - b));
      else if (gg <= r && gg <= b)
        s = W[i] * gg + (r <= b ? M[i] * (r - gg) + B[i] * (b - r) : M[i] * (b - gg) + R[i] * (r - b));
      else
        s = W[i] * b + (r <= b ? Yb[i] * (r - b) + G[i] * (gg - r) : Yb[i] * (gg - b) + R[i] * (r - gg));
      out[i] = s;
    }
  }
  // the solar disc (sunSpectrum): (sunD * (1, 1, -1)) . dir > sunThetaMax2
  // (the sum runs in every case, as `sky + black` does, so a -0 band of the
  // sky comes out +0 exactly as in the reference)
  float sd = m.sun_disc[0] * d[0] + m.sun_disc[1] * d[1] + (m.sun_disc[2] * -1.0f) * d[2];
  const bool disc = sd > m.stm;
  for (int i = 0; i < 16; i++) out[i] = out[i] + (disc ? m.sun_r[i] : 0.0f);
}

// evalSpd of an irregularly sampled SPD (Spectrum.hs:258-269)
static inline float skyEvalIrregular(const float* ls, const float* vs, int n, float l) {
  if (l <= ls[0]) return vs[0];
  if (l >= ls[n - 1]) return vs[n - 1];
  int lo = 0, hi = n - 1;
  for (;;) {
    int mid = (lo + hi) / 2;
    if (lo == mid) break;
    if (ls[mid] == l) {
      lo = mid;
      break;
    }
    if (ls[mid] < l)
      lo = mid;
    else
      hi = mid;
  }
  float t = (l - ls[lo]) / (ls[lo + 1] - ls[lo]);
  return (1.0f - t) * vs[lo] + t * vs[lo + 1];
}

// evalSpd of a regularly sampled SPD (Spectrum.hs:271-280)
static inline float skyEvalRegular(float l0, float l1, const float* a, int n, float l) {
  if (l <= l0) return a[0];
  if (l >= l1) return a[n - 1];
  float d1 = 1.0f / ((l1 - l0) / (float)(n - 1));
  float x = (l - l0) * d1;
  int b0 = (int)floorf(x);
  int b1 = b0 + 1 < n - 1 ? b0 + 1 : n - 1;
  float dx = x - (float)b0;
  return (1.0f - dx) * a[b0] + dx * a[b1];
}

// the sun's spectral curves (SunSky.hs:127-157): extraterrestrial solar
// irradiance, ozone, mixed-gas and water-vapour absorption
namespace sky_curves {
static const float kSol[38] = {
    165.5f, 162.3f, 211.2f, 258.8f, 258.2f, 242.3f, 267.6f, 296.6f, 305.4f, 300.6f,
    306.6f, 288.3f, 287.1f, 278.2f, 271.0f, 272.3f, 263.6f, 255.0f, 250.6f, 253.1f,
    253.5f, 251.3f, 246.3f, 241.7f, 236.8f, 232.1f, 228.2f, 223.4f, 219.7f, 215.3f,
    211.0f, 207.3f, 202.4f, 198.7f, 194.3f, 190.7f, 186.3f, 182.6f};
static const float kKoL[64] = {
    300, 305, 310, 315, 320, 325, 330, 335, 340, 345, 350, 355, 445, 450, 455, 460,
    465, 470, 475, 480, 485, 490, 495, 500, 505, 510, 515, 520, 525, 530, 535, 540,
    545, 550, 555, 560, 565, 570, 575, 580, 585, 590, 595, 600, 605, 610, 620, 630,
    640, 650, 660, 670, 680, 690, 700, 710, 720, 730, 740, 750, 760, 770, 780, 790};
static const float kKoA[64] = {
    10.0f,  4.8f,   2.7f,   1.35f,  0.8f,   0.380f, 0.160f, 0.075f, 0.04f,  0.019f, 0.007f,
    0.0f,   0.003f, 0.003f, 0.004f, 0.006f, 0.008f, 0.009f, 0.012f, 0.014f, 0.017f, 0.021f,
    0.025f, 0.03f,  0.035f, 0.04f,  0.045f, 0.048f, 0.057f, 0.063f, 0.07f,  0.075f, 0.08f,
    0.085f, 0.095f, 0.103f, 0.110f, 0.12f,  0.122f, 0.12f,  0.118f, 0.115f, 0.12f,  0.125f,
    0.130f, 0.12f,  0.105f, 0.09f,  0.079f, 0.067f, 0.057f, 0.048f, 0.036f, 0.028f, 0.023f,
    0.018f, 0.014f, 0.011f, 0.010f, 0.009f, 0.007f, 0.004f, 0.0f,   0.0f};
static const float kKgL[4] = {759, 760, 770, 771};
static const float kKgA[4] = {0.0f, 3.0f, 0.210f, 0.0f};
static const float kKwaL[13] = {689, 690, 700, 710, 720, 730, 740, 750, 760, 770, 780, 790, 800};
static const float kKwaA[13] = {0.0f,     0.160e-1f, 0.240e-1f, 0.125e-1f, 0.100e+1f,
                                0.870f,   0.610e-1f, 0.100e-2f, 0.100e-4f, 0.100e-4f,
                                0.600e-3f, 0.175e-1f, 0.360e-1f};
}  // namespace sky_curves

// host: the per-light constants of mkSunSkyLight east sunDir turbidity
// (SunSky.hs:12-65, 96-125) and the basis tables the evaluation needs
static inline void skyInit(const float east[3], const float sun_dir[3], float t, SkyModel& m) {
  const float kPiF = 3.14159274101257324f;
  memset(&m, 0, sizeof m);
  auto dot3 = [](const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
  auto normalize3 = [&](const float* v, float* o) {  // Math.hs:349-353
    float sl = dot3(v, v);
    if (sl != 0) {
      float il = 1.0f / sqrtf(sl);
      o[0] = v[0] * il;
      o[1] = v[1] * il;
      o[2] = v[2] * il;
    } else {
      o[0] = 0;
      o[1] = 1;
      o[2] = 0;
    }
  };
  auto cross3 = [](const float* u, const float* v, float* o) {  // Math.hs:336-339
    o[0] = u[1] * v[2] - u[2] * v[1];
    o[1] = -(u[0] * v[2] - u[2] * v[0]);
    o[2] = u[0] * v[1] - u[1] * v[0];
  };
  // basis = coordinateSystem' (normalize up) (normalize east) (Math.hs:427-432)
  const float up[3] = {0, 1, 0};
  float w[3], e[3], uu[3], vv[3], tmp[3];
  normalize3(up, w);
  normalize3(east, e);
  cross3(e, w, tmp);
  normalize3(tmp, uu);
  cross3(w, uu, vv);
  auto toLocal = [&](const float* v, float* o) {  // worldToLocal (Math.hs:439-441)
    o[0] = dot3(v, uu);
    o[1] = dot3(v, vv);
    o[2] = dot3(v, w);
  };
  float sdn[3], loc[3];
  normalize3(sun_dir, sdn);
  toLocal(sdn, loc);
  normalize3(loc, m.sky_sun);
  toLocal(sun_dir, loc);
  normalize3(loc, m.sun_disc);
  // initSky (SunSky.hs:45-65)
  float st = acosf(skyClamp(m.sky_sun[2], -1.0f, 1.0f));
  float st2 = st * st, st3 = st * st * st, t2 = t * t;
  float chi = (4.0f / 9.0f - t / 120.0f) * (kPiF - 2.0f * st);
  m.sun_theta = st;
  const float pY[5] = {0.17872f * t - 1.46303f, -0.35540f * t + 0.42749f, -0.02266f * t + 5.32505f,
                       0.12064f * t - 2.57705f, -0.06696f * t + 0.37027f};
  const float px[5] = {-0.01925f * t - 0.25922f, -0.06651f * t + 0.00081f, -0.00041f * t + 0.21247f,
                       -0.06409f * t - 0.89887f, -0.00325f * t + 0.04517f};
  const float py[5] = {-0.01669f * t - 0.26078f, -0.09495f * t + 0.00921f, -0.00792f * t + 0.21023f,
                       -0.04405f * t - 1.65369f, -0.01092f * t + 0.05291f};
  memcpy(m.pY, pY, sizeof pY);
  memcpy(m.px, px, sizeof px);
  memcpy(m.py, py, sizeof py);
  m.zY = ((4.04530f * t - 4.97100f) * tanf(chi) - 0.2155f * t + 2.4192f) * 1000.0f;
  m.zx = (0.00165f * st3 - 0.00374f * st2 + 0.00208f * st) * t2 +
         (-0.02902f * st3 + 0.06377f * st2 - 0.03202f * st + 0.00394f) * t +
         (0.11693f * st3 - 0.21196f * st2 + 0.06052f * st + 0.25885f);
  m.zy = (0.00275f * st3 - 0.00610f * st2 + 0.00316f * st) * t2 +
         (-0.04212f * st3 + 0.08970f * st2 - 0.04153f * st + 0.00515f) * t +
         (0.15346f * st3 - 0.26756f * st2 + 0.06669f * st + 0.26688f);
  // sunThetaMax2 (SunSky.hs:39-43)
  float sint2 = 6.955e5f / 1.496e8f;
  float om = 1.0f - sint2;
  m.stm = sqrtf(om < 0 ? 0.0f : om);
  for (int i = 0; i < 9; i++) m.s012[i] = __bling_f32(BLING_CIE_S012_XYZ_BITS[i]);
  for (int i = 0; i < 7 * 16; i++) m.illum[i] = __bling_f32(BLING_RGB_ILLUM_BITS[i]);
  // sunSpectrum' (SunSky.hs:96-125): fromSpd of the attenuated solar curve,
  // each band the mean of its two ends (avgSpd of a function, Spectrum.hs:316)
  if (m.sky_sun[2] < 0) return;  // below the horizon: black
  using namespace sky_curves;
  auto sf = [&](float l) {
    float mm = 1.0f / (cosf(st) + 0.000940f * powf(1.6386f - st, -1.253f));
    float tR = expf(-(mm * 0.008735f * powf(l / 1000.0f, -4.08f)));
    float beta = 0.04608365822050f * t - 0.04586025928522f;
    float tA = expf(-(mm * beta * powf(l / 1000.0f, -1.3f)));
    float tO = expf(-(mm * skyEvalIrregular(kKoL, kKoA, 64, l) * 0.35f));
    float kg = skyEvalIrregular(kKgL, kKgA, 4, l);
    float tG = expf(-(1.41f * kg * mm / powf(1.0f + 118.93f * kg * mm, 0.45f)));
    float kwa = skyEvalIrregular(kKwaL, kKwaA, 13, l);
    float tWA = expf(-(0.2385f * kwa * 2.0f * mm / powf(1.0f + 20.07f * kwa * 2.0f * mm, 0.45f)));
    return skyEvalRegular(380.0f, 750.0f, kSol, 38, l) * tR * tA * tO * tG * tWA;
  };
  for (int i = 0; i < 16; i++) {
    // lerp (i / bands) 400 700 (Math.hs:108-110)
    float a = (float)i / 16.0f, b = (float)(i + 1) / 16.0f;
    float l0 = (1.0f - a) * 400.0f + a * 700.0f, l1 = (1.0f - b) * 400.0f + b * 700.0f;
    m.sun_r[i] = (sf(l0) + sf(l1)) * 0.5f;
  }
}

}  // namespace bgpu
