// Upload of the shading data the path integrator needs: materials, meshes
// (vertices, indices, normals, uvs), per-primitive owners, shape emission and
// the light list in the reference's order (mkScene, Scene.hs:37-43), with
// the environment map's importance distribution (mkInfiniteAreaLight,
// Light.hs:72-82; mkDist2D, Montecarlo.hs:79-88).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "integrator.h"
#include "spectrum_tables.h"

namespace bgpu {
namespace {

float fbits(uint32_t b) {
  float f;
  memcpy(&f, &b, 4);
  return f;
}

// sY on the host (Spectrum.hs:371-373), for the environment map's distribution
float sYHost(const float* s) {
  float acc = 0.0f;
  for (int i = 0; i < 16; i++) acc = acc + s[i] * fbits(BLING_CIE_Y_BITS[i]);
  return acc / fbits(BLING_CIE_Y_SUM_BITS);
}
// mkDist1D (Montecarlo.hs:40-48)
void mkDist1D(const float* func, int n, float* cdf, float& fi) {
  std::vector<float> i(n + 1);
  i[0] = 0;
  for (int k = 0; k < n; k++) i[k + 1] = i[k] + func[k] / (float)n;
  fi = i[n];
  for (int k = 0; k <= n; k++) cdf[k] = fi != 0 ? i[k] / fi : (float)k / (float)n;
}

}  // namespace

#define RET_CUDA(call)                                                      \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) {                                                \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);             \
      return e_ == cudaErrorMemoryAllocation ? BLING_ERR_OOM : BLING_ERR_CUDA; \
    }                                                                       \
  } while (0)

int integrator_upload_scene(cudaStream_t stream, const bling_scene_desc& d,
                            const std::vector<int32_t>& order, const std::vector<int32_t>& prim_owner,
                            const std::vector<int32_t>& prim_tri, const std::vector<DShape>& shapes,
                            const std::vector<int32_t>& shape_light, std::vector<void*>& owned,
                            DevShading& out, std::string& err) {
  out = DevShading{};
  size_t bytes = 0;
  auto up = [&](const void* host, size_t nbytes, void** dptr) -> int {
    *dptr = nullptr;
    if (nbytes == 0) return BLING_OK;
    RET_CUDA(cudaMalloc(dptr, nbytes));
    owned.push_back(*dptr);
    bytes += nbytes;
    RET_CUDA(cudaMemcpyAsync(*dptr, host, nbytes, cudaMemcpyHostToDevice, stream));
    return BLING_OK;
  };
  int rc;
  // materials
  std::vector<DMaterial> mats(d.n_materials);
  for (int i = 0; i < d.n_materials; i++) {
    const bling_material& m = d.materials[i];
    DMaterial& o = mats[i];
    o.kind = m.kind;
    o.sigma = m.sigma;
    o.rough = m.roughness;
    o.ior = m.ior;
    memcpy(o.kd, m.kd, 64);
    memcpy(o.ks, m.ks, 64);
    memcpy(o.kt, m.kt, 64);
    memcpy(o.eta, m.eta, 64);
    memcpy(o.k, m.k, 64);
    o.kd_tex = m.kd_texture;
    memcpy(o.kd_par, m.kd_tex_params, 36);
    memcpy(o.kd2, m.kd2, 64);
    o.textured = m.bump != 0;
    for (int k = 0; k < 8; k++) {
      o.tex[k] = m.tex[k];
      o.textured |= m.tex[k] != 0;
    }
    o.bump = m.bump;
    if (!o.textured) deriveMaterialSpectra(o);  // textured ones derive per hit
    out.textured |= o.textured;
  }
  // texture nodes, with the images and gradients they read
  if (d.n_textures > 0) {
    std::vector<DTex> tex(d.n_textures);
    for (int i = 0; i < d.n_textures; i++) {
      const bling_texture& t = d.textures[i];
      DTex& o = tex[i];
      memset(&o, 0, sizeof o);
      o.kind = t.kind;
      o.a = t.a;
      o.b = t.b;
      o.c = t.c;
      o.ivalue = t.ivalue;
      o.map_kind = t.map_kind;
      memcpy(o.map, t.map, sizeof o.map);
      memcpy(o.p, t.p, sizeof o.p);
      memcpy(o.spectrum, t.spectrum, sizeof o.spectrum);
      o.width = t.width;
      o.height = t.height;
      std::vector<float> data;
      if (t.kind == BLING_TEXN_GRADIENT) {
        // mkGradient: the steps sorted by position, ties in their given order
        std::vector<int> idx(t.ivalue);
        for (int k = 0; k < t.ivalue; k++) idx[k] = k;
        std::stable_sort(idx.begin(), idx.end(),
                         [&](int x, int y) { return t.data[17 * x] < t.data[17 * y]; });
        data.resize((size_t)17 * t.ivalue);
        for (int k = 0; k < t.ivalue; k++) memcpy(&data[17 * k], t.data + 17 * idx[k], 68);
      } else if (t.kind == BLING_TEXN_IMAGE) {
        // pixelSpectrum: rgbToSpectrumRefl (unGamma (r/255, g/255, b/255))
        // (Texture.hs:87-89, Spectrum.hs:118-120), once per pixel
        size_t n = (size_t)t.width * t.height;
        data.resize(16 * n);
        for (size_t k = 0; k < n; k++) {
          float c[3];
          for (int j = 0; j < 3; j++) c[j] = powf((float)t.pixels[3 * k + j] / 255.0f, 2.2f);
          bling_rgb_to_spectrum(0, c[0], c[1], c[2], &data[16 * k]);
        }
      } else if (t.kind == BLING_TEXN_IMAGE_SCALAR) {  // getPixelScalar: pixel / 255
        size_t n = (size_t)t.width * t.height;
        data.resize(n);
        for (size_t k = 0; k < n; k++) data[k] = (float)t.pixels[k] / 255.0f;
      }
      if (!data.empty()) {
        void* p;
        if ((rc = up(data.data(), data.size() * 4, &p))) return rc;
        RET_CUDA(cudaStreamSynchronize(stream));  // `data` is a temporary
        o.data = (const float*)p;
      }
    }
    void* dt;
    if ((rc = up(tex.data(), tex.size() * sizeof(DTex), &dt))) return rc;
    RET_CUDA(cudaStreamSynchronize(stream));
    out.tex = (const DTex*)dt;
  }
  void* dm;
  if ((rc = up(mats.data(), mats.size() * sizeof(DMaterial), &dm))) return rc;
  out.materials = (const DMaterial*)dm;
  out.n_materials = d.n_materials;
  // meshes
  std::vector<DMesh> meshes(d.n_meshes);
  for (int i = 0; i < d.n_meshes; i++) {
    const bling_mesh_desc& m = d.meshes[i];
    DMesh& o = meshes[i];
    memset(&o, 0, sizeof o);
    void* p;
    if ((rc = up(m.vertices, (size_t)m.n_vertices * 12, &p))) return rc;
    o.verts = (const float*)p;
    if ((rc = up(m.indices, (size_t)m.n_indices * 4, &p))) return rc;
    o.idx = (const int32_t*)p;
    if (m.normals) {
      if ((rc = up(m.normals, (size_t)m.n_vertices * 12, &p))) return rc;
      o.normals = (const float*)p;
    }
    if (m.uvs) {
      if ((rc = up(m.uvs, (size_t)m.n_vertices * 8, &p))) return rc;
      o.uvs = (const float*)p;
    }
    o.material = m.material;
  }
  void* dmesh;
  if ((rc = up(meshes.data(), meshes.size() * sizeof(DMesh), &dmesh))) return rc;
  out.meshes = (const DMesh*)dmesh;
  // per-primitive owner
  std::vector<int2> info(prim_owner.size());
  for (size_t i = 0; i < info.size(); i++) info[i] = make_int2(prim_owner[i], prim_tri[i]);
  void* dinfo;
  if ((rc = up(info.data(), info.size() * sizeof(int2), &dinfo))) return rc;
  out.prim_info = (const int2*)dinfo;
  // the primitive ID of every shape
  std::vector<int32_t> shape_prim(std::max<size_t>(1, d.n_shapes), -1);
  for (size_t i = 0; i < prim_owner.size(); i++)
    if (prim_owner[i] < 0) shape_prim[~prim_owner[i]] = (int32_t)i;
  void* dsp;
  if ((rc = up(shape_prim.data(), shape_prim.size() * 4, &dsp))) return rc;
  out.shape_prim = (const int32_t*)dsp;
  // shape emission
  std::vector<float> em(16 * std::max<size_t>(1, d.n_shapes), 0.0f);
  for (int i = 0; i < d.n_shapes; i++) memcpy(&em[16 * i], d.shapes[i].emission, 64);
  void* dem;
  if ((rc = up(em.data(), em.size() * 4, &dem))) return rc;
  out.shape_emission = (const float*)dem;
  // lights: the non-geometric ones, then the emissive shapes in primitive order
  std::vector<DLight> lights;
  for (int i = 0; i < d.n_lights; i++) {
    const bling_light_desc& l = d.lights[i];
    DLight o;
    memset(&o, 0, sizeof o);
    o.kind = l.kind;
    o.shape = -1;
    memcpy(o.spec, l.spectrum, 64);
    memcpy(o.vec, l.vec, 12);
    memcpy(o.w2l, l.w2l, 64);
    memcpy(o.l2w, l.l2w, 64);
    if (l.kind == BLING_LIGHT_INFINITE || l.kind == BLING_LIGHT_SUNSKY) {
      const bool sky = l.kind == BLING_LIGHT_SUNSKY;
      int w = sky ? kSkyMapW : l.env_w, h = sky ? kSkyMapH : l.env_h;
      if (!sky && (w <= 0 || h <= 0 || !l.env)) {
        err = "infinite light without an environment map";
        return BLING_ERR_INVALID_ARG;
      }
      o.kind = BLING_LIGHT_INFINITE;  // one kind on the device; `sky` tells the maps apart
      o.env_w = w;
      o.env_h = h;
      void* p;
      SkyModel model;
      if (sky) {  // mkSunSkyLight east sunDir turbidity (SunSky.hs:12-24)
        skyInit(l.east, l.vec, l.turbidity, model);
        if ((rc = up(&model, sizeof model, &p))) return rc;
        o.sky = (const SkyModel*)p;
      } else {
        if ((rc = up(l.env, (size_t)w * h * 64, &p))) return rc;
        o.env = (const float*)p;
      }
      // mkInfiniteAreaLight's Dist2D over sY of the map at each raster
      // position (x / w, y / h) (Light.hs:72-82, Montecarlo.hs:79-88)
      std::vector<float> func((size_t)w * h), cdf((size_t)h * (w + 1)), cint(h), mcdf(h + 1);
      for (int v = 0; v < h; v++) {
        for (int u = 0; u < w; u++) {
          float uu = (float)u / (float)w, vv = (float)v / (float)h;
          if (sky) {
            float texel[16];
            skyEval(model, uu, vv, texel);
            func[(size_t)v * w + u] = sYHost(texel);
          } else {
            int x = std::max(0, std::min(w - 1, (int)floorf(uu * (float)w)));
            int y = std::max(0, std::min(h - 1, (int)floorf(vv * (float)h)));
            func[(size_t)v * w + u] = sYHost(l.env + 16 * ((size_t)y * w + x));
          }
        }
        mkDist1D(&func[(size_t)v * w], w, &cdf[(size_t)v * (w + 1)], cint[v]);
      }
      float mint;
      mkDist1D(cint.data(), h, mcdf.data(), mint);
      if ((rc = up(func.data(), func.size() * 4, &p))) return rc;
      o.cond_func = (const float*)p;
      if ((rc = up(cdf.data(), cdf.size() * 4, &p))) return rc;
      o.cond_cdf = (const float*)p;
      if ((rc = up(cint.data(), cint.size() * 4, &p))) return rc;
      o.cond_int = (const float*)p;
      if ((rc = up(mcdf.data(), mcdf.size() * 4, &p))) return rc;
      o.marg_cdf = (const float*)p;
      o.marg_int = mint;
    }
    lights.push_back(o);
  }
  for (int32_t v : order) {
    if (v >= 0 || shape_light[~v] < 0) continue;
    DLight o;
    memset(&o, 0, sizeof o);
    o.kind = DLIGHT_AREA;
    o.shape = ~v;
    lights.push_back(o);
  }
  void* dl;
  if ((rc = up(lights.data(), lights.size() * sizeof(DLight), &dl))) return rc;
  out.lights = (const DLight*)dl;
  out.n_lights = (int32_t)lights.size();
  out.camera = d.camera;
  out.bytes = bytes;
  (void)shapes;
  return BLING_OK;
}

}  // namespace bgpu
