// Wavefront path integrator: host-side interface (integrator.cu).
#pragma once
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bling_gpu.h"
#include "internal.h"
#include "sunsky.h"

namespace bgpu {

struct DMaterial {
  int kind;
  float sigma, rough, ior;
  float kd[16], ks[16], kt[16], eta[16], k[16];
  int kd_tex;           // BLING_TEX_*
  float kd_par[9];      // the texture's parameters (bling_material.kd_tex_params)
  float kd2[16];        // the texture's second spectrum
  int tex[8];           // bling_material.tex: texture node + 1 per parameter slot, 0 constant
  int bump;             // displacement node + 1, 0 none
  int textured;         // any tex or bump: the derived spectra are made per hit
};

// a texture node on the device (bling_texture; texture.cuh evaluates it)
struct DTex {
  int kind, a, b, c, ivalue, map_kind;
  float map[16];
  float p[4];
  float spectrum[16];
  // gradient: ivalue steps of 17 floats (position, spectrum), sorted by
  // position; image: width x height spectra (pixelSpectrum of each pixel,
  // Texture.hs:87-89); grey image: width x height values (pixel / 255)
  const float* data;
  int width, height;
};

// Spectra a material derives from its constant parameters, once at upload
// (the reference derives them per hit from constant textures: same values).
//  * shiny metal (Material.hs:98-109): eta/k <- frApproxEta/frApproxK of ks
//    for the microfacet lobe, kd/kt <- frApproxEta/frApproxK of kr (given in
//    kd) for the specular lobe (Fresnel.hs:72-78);
//  * translucent matte (Material.hs:43-53): kd <- r = sClamp 0 1 kr,
//    kt <- t = sClamp 0 1 kt * (white - r).
// Haskell's clamp, min and max order (max lo (min hi x)) is kept.  A
// textured material derives them per hit, after its textures are evaluated.
BLING_HD inline float ghcClamp(float x, float lo, float hi) {
  float m = hi <= x ? hi : x;  // min hi x
  return lo <= m ? m : lo;     // max lo m
}
BLING_HD inline void deriveMaterialSpectra(DMaterial& m) {
  if (m.kind == BLING_MAT_SHINY_METAL) {
    float kr[16];
    for (int i = 0; i < 16; i++) kr[i] = m.kd[i];
    for (int i = 0; i < 16; i++) {
      float rs = sqrtf(ghcClamp(m.ks[i], 0.0f, 0.999f));
      float refl = ghcClamp(m.ks[i], 0.0f, 0.999f);
      m.eta[i] = (1.0f + rs) / (1.0f - rs);
      m.k[i] = sqrtf(refl / (1.0f - refl)) * 2.0f;
      float rr = sqrtf(ghcClamp(kr[i], 0.0f, 0.999f));
      float reflr = ghcClamp(kr[i], 0.0f, 0.999f);
      m.kd[i] = (1.0f + rr) / (1.0f - rr);
      m.kt[i] = sqrtf(reflr / (1.0f - reflr)) * 2.0f;
    }
  } else if (m.kind == BLING_MAT_TRANS_MATTE) {
    for (int i = 0; i < 16; i++) {
      float r = ghcClamp(m.kd[i], 0.0f, 1.0f);
      m.kt[i] = ghcClamp(m.kt[i], 0.0f, 1.0f) * (1.0f - r);
      m.kd[i] = r;
    }
  } else if (m.kind == BLING_MAT_SUBSTRATE) {
    // mkSubstrate (Material.hs:111-127): rd, rs, ra = sClamp 0 1 of kd, ks,
    // ka (in kt); mkAnisotropic (1 / u) (1 / v) with u, v = max 0 of the
    // roughnesses; the exponents go to rough (ex) and sigma (ey)
    for (int i = 0; i < 16; i++) {
      m.kd[i] = ghcClamp(m.kd[i], 0.0f, 1.0f);
      m.kd2[i] = ghcClamp(m.kd2[i], 0.0f, 1.0f);
      m.ks[i] = ghcClamp(m.ks[i], 0.0f, 1.0f);
      m.kt[i] = ghcClamp(m.kt[i], 0.0f, 1.0f);
    }
    float u = 0.0f <= m.rough ? m.rough : 0.0f, v = 0.0f <= m.sigma ? m.sigma : 0.0f;
    float ex = 1.0f / u, ey = 1.0f / v;
    m.rough = (ex > 10000 || ex != ex) ? 10000.0f : ex;  // fixExponent (Microfacet.hs:126-128)
    m.sigma = (ey > 10000 || ey != ey) ? 10000.0f : ey;
  }
}

struct DMesh {
  const float* verts;   // 3 per vertex (world space)
  const int32_t* idx;   // 3 per triangle
  const float* normals; // 3 per vertex or null
  const float* uvs;     // 2 per vertex or null
  int32_t material;
  int32_t pad;
};

enum { DLIGHT_DIRECTIONAL = 0, DLIGHT_POINT = 1, DLIGHT_INFINITE = 2, DLIGHT_AREA = 100 };

struct DLight {
  int kind;
  int shape;   // area lights
  int env_w, env_h;
  float spec[16];
  float vec[3];
  float w2l[16], l2w[16];
  const float* env;        // env_h * env_w * 16
  const float* cond_func;  // env_h * env_w
  const float* cond_cdf;   // env_h * (env_w + 1)
  const float* cond_int;   // env_h
  const float* marg_cdf;   // env_h + 1
  float marg_int;
  float pad;
  // sun/sky (BLING_LIGHT_SUNSKY): the map is this model, evaluated at
  // continuous (u, v); env is null and env_w x env_h only size the Dist2D
  const SkyModel* sky;
};

struct DevShading {
  const DMaterial* materials;
  const DTex* tex;  // the scene's texture nodes
  int textured;     // some material is textured: shading kernels take the textured variant
  const DMesh* meshes;
  const int2* prim_info;   // (owner, triangle): owner >= 0 mesh, < 0 ~shape
  const float* shape_emission;  // 16 per shape
  const DLight* lights;
  int32_t n_lights;
  int32_t n_materials;
  const int32_t* shape_prim;  // per shape: its primitive ID (MIS queries rank against it)
  bling_camera_desc camera;
  size_t bytes;
};

struct PassResult {
  uint64_t rays_closest, rays_any, path_samples, nonfinite, degenerate;
  // the pass's first dropped (NaN/Inf) sample: pixel and sample number, or
  // nf_x = -1 when none was dropped
  int32_t nf_x = -1, nf_y = -1, nf_n = -1;
};

// Device buffer reused across passes (grow-only), owned by a context: the
// path slots, queues and counters of one wavefront chunk, laid out by
// integrator.cu.
struct IntegratorWorkspace {
  size_t capacity = 0;  // path slots
  void* buffer = nullptr;
};

int integrator_upload_scene(cudaStream_t stream, const bling_scene_desc& d,
                            const std::vector<int32_t>& order, const std::vector<int32_t>& prim_owner,
                            const std::vector<int32_t>& prim_tri, const std::vector<DShape>& shapes,
                            const std::vector<int32_t>& shape_light, std::vector<void*>& owned,
                            DevShading& out, std::string& err);

// bin_box (6 floats: the scene's world bounds lo.xyz, hi.xyz) turns on ray
// binning of the bounces after the camera's (BLING_FLAG_BIN_RAYS); null: off
int integrator_render_pass(cudaStream_t stream, const DevAccel& A, const DevShading& S,
                           const bling_render_params& p, uint64_t pass, float* d_film, int fw,
                           int fh, IntegratorWorkspace& ws, PassResult& res, std::string& err,
                           const float* bin_box = nullptr);

void integrator_workspace_free(IntegratorWorkspace& ws);

// One pass whose path state lives in a file-scope device array (no device
// allocation); at most integrator_noalloc_max_samples() path samples.
int integrator_render_pass_noalloc(cudaStream_t stream, const DevAccel& A, const DevShading& S,
                                   const bling_render_params& p, uint64_t pass, float* d_film,
                                   int fw, int fh, PassResult& res, std::string& err);
size_t integrator_noalloc_max_samples();

}  // namespace bgpu
