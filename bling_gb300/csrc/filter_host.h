// Pixel filters evaluated on the host for the 16x16 filter table
// (evalFilter, Filter.hs:68-96; mkTableFilter, Image.hs:48-61).
#pragma once
#include <cmath>

#include "../../include/bling_gpu.h"
#include "dmath.cuh"

namespace bgpu {

static inline float evalFilterHost(int kind, const float* fp, float x, float y) {
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


// the table: entry [y * 16 + x] = filter at ((x + 0.5) fw / 16, (y + 0.5) fh / 16)
static inline void filterTableHost(int kind, const float* fp, float fw, float fh, float* tbl) {
  for (int y = 0; y < 16; y++) {
    float fy = ((float)y + 0.5f) * fh / 16.0f;
    for (int x = 0; x < 16; x++) {
      float fx = ((float)x + 0.5f) * fw / 16.0f;
      tbl[y * 16 + x] = evalFilterHost(kind, fp, fx, fy);
    }
  }
}

}  // namespace bgpu
