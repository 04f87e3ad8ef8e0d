// C ABI of the GB300 path-tracing core (include/bling_gpu.h).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bling_gpu.h"
#include "batch.h"
#include "bvh.h"
#include "bvh_gpu.h"
#include "handles.h"
#include "integrator.h"
#include "internal.h"
#include "spectrum_tables.h"

using namespace bgpu;

static std::atomic<uint64_t> g_scene_serial{0};

namespace {

int set_err(bling_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CK(ctx, call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return set_err((ctx), BLING_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                     __FILE__, __LINE__);                                               \
  } while (0)

int ensure_scratch(bling_ctx* c, size_t bytes) {
  if (c->scratch_bytes >= bytes) return BLING_OK;
  if (c->d_scratch) cudaFree(c->d_scratch);
  c->d_scratch = nullptr;
  c->scratch_bytes = 0;
  size_t want = std::max(bytes, c->scratch_bytes * 2);
  cudaError_t e = cudaMalloc(&c->d_scratch, want);
  if (e != cudaSuccess) {
    e = cudaMalloc(&c->d_scratch, bytes);
    want = bytes;
  }
  if (e != cudaSuccess)
    return set_err(c, e == cudaErrorMemoryAllocation ? BLING_ERR_OOM : BLING_ERR_CUDA,
                   "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  c->scratch_bytes = want;
  return BLING_OK;
}

// ---- host-buffer ray queries, chunked so that copies overlap traversal
//
// The rays (SoA, 8 floats per ray) are copied in, traced and their results
// copied out chunk by chunk through kPipeBuffers staging buffers: while a
// kernel traces chunk k, chunk k+1 is copied in on one copy stream and chunk
// k-1's results are copied out on another.  Consecutive chunks are traced on
// two compute streams in turn (the context's and compute2), each buffer with
// its own work counter (d_counter[1 + buffer]), so that a chunk's blocks take
// the SMs its predecessor's last warps leave idle instead of waiting for the
// whole predecessor.
constexpr int kPipeBuffers = 3;
constexpr size_t kPipeChunk = size_t(1) << 21;  // rays per chunk
static_assert(1 + kPipeBuffers <= 256 / 8, "the context's 256-byte counter block holds the chunk counters");

struct QueryOut {
  void* host;
  size_t bytes_per_ray;
};

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

int ensure_pipeline(bling_ctx* c) {
  if (c->copy_in) return BLING_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&c->copy_in, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy_out, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->compute2, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_start, cudaEventDisableTiming);
  for (int b = 0; b < kPipeBuffers && e == cudaSuccess; b++) {
    e = cudaEventCreateWithFlags(&c->ev_in[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_run[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_out[b], cudaEventDisableTiming);
  }
  if (e != cudaSuccess)
    return set_err(c, BLING_ERR_CUDA, "copy stream creation: %s", cudaGetErrorString(e));
  return BLING_OK;
}

void destroy_pipeline(bling_ctx* c) {
  if (c->copy_in) cudaStreamDestroy(c->copy_in);
  if (c->copy_out) cudaStreamDestroy(c->copy_out);
  if (c->compute2) cudaStreamDestroy(c->compute2);
  if (c->ev_start) cudaEventDestroy(c->ev_start);
  for (int b = 0; b < kPipeBuffers; b++) {
    if (c->ev_in[b]) cudaEventDestroy(c->ev_in[b]);
    if (c->ev_run[b]) cudaEventDestroy(c->ev_run[b]);
    if (c->ev_out[b]) cudaEventDestroy(c->ev_out[b]);
  }
  c->copy_in = c->copy_out = c->compute2 = nullptr;
}

// launch(d_rays, count, d_outs, d_counter, stream) enqueues the query kernel
// of one chunk on `stream` with work counter d_counter; outs[j] receives
// bytes_per_ray bytes per ray.  Called with c->mu held; returns once every
// result is in host memory.
template <class Launch>
int pipelined_query(bling_ctx* c, const float* rays, size_t n, const QueryOut* outs, int n_outs,
                    Launch launch) {
  const size_t chunk = std::min(n, kPipeChunk);
  size_t slot = align256(32 * chunk);
  for (int j = 0; j < n_outs; j++) slot += align256(outs[j].bytes_per_ray * chunk);
  int rc = ensure_scratch(c, kPipeBuffers * slot);
  if (rc) return rc;
  rc = ensure_pipeline(c);
  if (rc) return rc;
  // the copy streams start after the work already queued on the context's stream
  CK(c, cudaEventRecord(c->ev_start, c->stream));
  CK(c, cudaStreamWaitEvent(c->copy_in, c->ev_start, 0));
  for (size_t i = 0, k = 0; i < n; i += chunk, k++) {
    const int b = (int)(k % kPipeBuffers);
    const size_t cn = std::min(chunk, n - i);
    char* base = (char*)c->d_scratch + b * slot;
    float* d_r = (float*)base;
    void* d_out[4] = {nullptr, nullptr, nullptr, nullptr};
    size_t off = align256(32 * chunk);
    for (int j = 0; j < n_outs; j++) {
      d_out[j] = base + off;
      off += align256(outs[j].bytes_per_ray * chunk);
    }
    // the buffer's previous results must be out before new rays come in
    if (k >= (size_t)kPipeBuffers) CK(c, cudaStreamWaitEvent(c->copy_in, c->ev_out[b], 0));
    // the chunk's slice of each of the 8 ray rows (o, d, tmin, tmax)
    for (int row = 0; row < 8; row++)
      CK(c, cudaMemcpyAsync(d_r + row * cn, rays + row * n + i, cn * sizeof(float),
                            cudaMemcpyHostToDevice, c->copy_in));
    CK(c, cudaEventRecord(c->ev_in[b], c->copy_in));
    cudaStream_t ks = (k & 1) ? c->compute2 : c->stream;
    CK(c, cudaStreamWaitEvent(ks, c->ev_in[b], 0));
    CK(c, launch(d_r, (int64_t)cn, d_out, c->d_counter + 1 + b, ks));
    CK(c, cudaEventRecord(c->ev_run[b], ks));
    CK(c, cudaStreamWaitEvent(c->copy_out, c->ev_run[b], 0));
    for (int j = 0; j < n_outs; j++)
      CK(c, cudaMemcpyAsync((char*)outs[j].host + i * outs[j].bytes_per_ray, d_out[j],
                            cn * outs[j].bytes_per_ray, cudaMemcpyDeviceToHost, c->copy_out));
    CK(c, cudaEventRecord(c->ev_out[b], c->copy_out));
  }
  // every copy-out follows its chunk's kernel; the last one follows them all
  CK(c, cudaStreamSynchronize(c->copy_out));
  return BLING_OK;
}

template <class T>
int upload(bling_ctx* c, std::vector<void*>& owned, const T* host, size_t count, T** out) {
  *out = nullptr;
  if (count == 0) return BLING_OK;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, count * sizeof(T));
  if (e != cudaSuccess)
    return set_err(c, e == cudaErrorMemoryAllocation ? BLING_ERR_OOM : BLING_ERR_CUDA,
                   "cudaMalloc(%zu): %s", count * sizeof(T), cudaGetErrorString(e));
  owned.push_back(p);
  CK(c, cudaMemcpyAsync(p, host, count * sizeof(T), cudaMemcpyHostToDevice, c->stream));
  *out = (T*)p;
  return BLING_OK;
}

float fbits(uint32_t b) {
  float f;
  memcpy(&f, &b, 4);
  return f;
}

// objectBounds (Shape.hs:295-311) and transBox (Transform.hs:281-292)
void shape_world_bounds(const bling_shape_desc& s, float lo[3], float hi[3]) {
  float olo[3], ohi[3];
  const float* p = s.params;
  switch (s.kind) {
    case BLING_SHAPE_BOX:
      for (int k = 0; k < 3; k++) {
        olo[k] = p[k];
        ohi[k] = p[3 + k];
      }
      break;
    case BLING_SHAPE_CYLINDER:
      olo[0] = olo[1] = -p[0];
      ohi[0] = ohi[1] = p[0];
      olo[2] = p[1];
      ohi[2] = p[2];
      break;
    case BLING_SHAPE_DISK:
      olo[0] = olo[1] = -p[1];
      ohi[0] = ohi[1] = p[1];
      olo[2] = ohi[2] = p[0];
      break;
    case BLING_SHAPE_QUAD:
      olo[0] = -p[0];
      olo[1] = -p[1];
      ohi[0] = p[0];
      ohi[1] = p[1];
      olo[2] = ohi[2] = 0;
      break;
    default:
      for (int k = 0; k < 3; k++) {
        olo[k] = -p[0];
        ohi[k] = p[0];
      }
  }
  for (int k = 0; k < 3; k++) {
    lo[k] = INFINITY;
    hi[k] = -INFINITY;
  }
  for (int c = 0; c < 8; c++) {
    V3 q{(c & 4) ? ohi[0] : olo[0], (c & 2) ? ohi[1] : olo[1], (c & 1) ? ohi[2] : olo[2]};
    V3 w = transPoint(s.o2w, q);
    float wv[3] = {w.x, w.y, w.z};
    for (int k = 0; k < 3; k++) {
      lo[k] = std::min(lo[k], wv[k]);
      hi[k] = std::max(hi[k], wv[k]);
    }
  }
}

}  // namespace

// sampler/integrator/filter parameters of a pass (the checks of
// bling_render_pass); touches no shared state, so any thread may call it
int bgpu::validate_render_params(const bling_render_params* p, std::string& err) {
  char buf[160];
  auto fail = [&](const char* msg) {
    err = msg;
    return BLING_ERR_INVALID_ARG;
  };
  if (p->width <= 0 || p->height <= 0) {
    snprintf(buf, sizeof buf, "invalid image size %dx%d", p->width, p->height);
    return fail(buf);
  }
  if (p->strata_x <= 0 || p->strata_y <= 0 || p->max_depth < 0 || p->sample_depth < 0 ||
      p->strata_x * p->strata_y > 4096)
    return fail("invalid sampler/integrator parameters");
  if (p->filter_kind < BLING_FILTER_BOX || p->filter_kind > BLING_FILTER_TRIANGLE) {
    snprintf(buf, sizeof buf, "unknown filter kind %d", p->filter_kind);
    return fail(buf);
  }
  if (p->sampler_kind != BLING_SAMPLER_STRATIFIED && p->sampler_kind != BLING_SAMPLER_RANDOM) {
    snprintf(buf, sizeof buf, "unknown sampler kind %d", p->sampler_kind);
    return fail(buf);
  }
  if (p->reserved != 0) return fail("bling_render_params.reserved must be 0");
  return BLING_OK;
}

int bgpu::check_render_params(bling_ctx* c, const bling_render_params* p) {
  std::string err;
  int rc = validate_render_params(p, err);
  if (rc != BLING_OK) return set_err(c, rc, "%s", err.c_str());
  return BLING_OK;
}

// acc += pass; pass = 0 (the FP64 accumulator of a BLING_FILM_FP64 film)
__global__ void k_film_fold(float* __restrict__ pass, double* __restrict__ acc, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    float v = pass[i];
    if (v != 0.0f) {
      acc[i] += (double)v;
      pass[i] = 0.0f;
    }
  }
}

static cudaError_t film_fold(bling_film* f, cudaStream_t stream) {
  if (!f->d_acc) return cudaSuccess;
  size_t n = (size_t)f->width * f->height * 4;
  unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 4096);
  k_film_fold<<<grid, 256, 0, stream>>>(f->d_film, f->d_acc, n);
  return cudaGetLastError();
}

extern "C" {

int bling_abi_version(void) { return BLING_ABI_VERSION; }

int bling_ctx_create(bling_ctx** out, const bling_opts* opts) {
  if (!out) return BLING_ERR_INVALID_ARG;
  *out = nullptr;
  std::unique_ptr<bling_ctx> c(new bling_ctx());
  if (opts) c->opts = *opts;
  c->device = c->opts.device;
  {
    const uint32_t f = c->opts.flags;
    const int layouts = ((f & BLING_FLAG_WIDE_BVH) ? 1 : 0) + ((f & BLING_FLAG_GPU_BVH) ? 1 : 0) +
                        ((f & BLING_FLAG_COMPACT_BVH) ? 1 : 0);
    if (layouts > 1 || (f & ~(BLING_FLAG_WIDE_BVH | BLING_FLAG_GPU_BVH | BLING_FLAG_COMPACT_BVH |
                              BLING_FLAG_BIN_RAYS))) {
      set_err(c.get(), BLING_ERR_INVALID_ARG,
              "bling_opts.flags: at most one of BLING_FLAG_WIDE_BVH, BLING_FLAG_GPU_BVH and "
              "BLING_FLAG_COMPACT_BVH, and no unknown flags");
      *out = c.release();
      return BLING_ERR_INVALID_ARG;
    }
  }
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev <= 0) {
    // keep the context so the caller can read the message
    set_err(c.get(), BLING_ERR_CUDA, "no usable CUDA device: %s", cudaGetErrorString(e));
    *out = c.release();
    return BLING_ERR_CUDA;
  }
  if (c->device < 0 || c->device >= ndev) {
    set_err(c.get(), BLING_ERR_INVALID_ARG, "device %d out of range (%d devices)", c->device, ndev);
    *out = c.release();
    return BLING_ERR_INVALID_ARG;
  }
  e = cudaSetDevice(c->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_counter, 256);
  c->stream = c->own_stream;
  if (e != cudaSuccess) {
    set_err(c.get(), BLING_ERR_CUDA, "stream creation failed: %s", cudaGetErrorString(e));
    *out = c.release();
    return BLING_ERR_CUDA;
  }
  *out = c.release();
  return BLING_OK;
}

void bling_ctx_destroy(bling_ctx* c) {
  if (!c) return;
  {
    std::lock_guard<std::mutex> g(c->mu);
    if (c->own_stream) {
      cudaSetDevice(c->device);
      cudaStreamSynchronize(c->stream);
      cudaStreamSynchronize(c->own_stream);
      cudaStreamDestroy(c->own_stream);
    }
    if (c->copy_out) cudaStreamSynchronize(c->copy_out);
    destroy_pipeline(c);
    if (c->d_scratch) cudaFree(c->d_scratch);
    if (c->d_counter) cudaFree(c->d_counter);
    integrator_workspace_free(c->ws);
    light_workspace_free(c->lt_ws);
    sppm_workspace_free(c->sp_ws);
  }
  delete c;
}

const char* bling_last_error(bling_ctx* c) { return c ? c->err.c_str() : "null context"; }

int bling_ctx_set_stream(bling_ctx* c, void* stream) {
  if (!c) return BLING_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (!c->own_stream) return set_err(c, BLING_ERR_STATE, "context has no device");
  CK(c, cudaSetDevice(c->device));
  CK(c, cudaStreamSynchronize(c->stream));
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return BLING_OK;
}

// ---- texture expressions: node kinds, children before parents and of the
// right value type, mappings, sizes, depth; material slots name nodes of the
// slot's type
static bool tex_is_scalar(int kind) { return kind >= BLING_TEXN_SCALAR && kind <= BLING_TEXN_IMAGE_SCALAR; }
static bool tex_is_spectrum(int kind) { return kind >= BLING_TEXN_CONSTANT && kind <= BLING_TEXN_IMAGE; }
static bool check_textures(const bling_scene_desc& d, std::string& err) {
  char buf[160];
  auto fail = [&](int i, const char* what) {
    snprintf(buf, sizeof buf, "texture %d: %s", i, what);
    err = buf;
    return false;
  };
  if (d.n_textures < 0 || (d.n_textures > 0 && !d.textures)) {
    err = "bad texture array";
    return false;
  }
  std::vector<int> depth(d.n_textures, 1);
  for (int i = 0; i < d.n_textures; i++) {
    const bling_texture& t = d.textures[i];
    if (!tex_is_scalar(t.kind) && !tex_is_spectrum(t.kind)) return fail(i, "unknown kind");
    // the children each kind reads: 'S' spectrum, 'F' scalar, '-' none
    const char* want = "---";
    switch (t.kind) {
      case BLING_TEXN_BLEND: want = "SSF"; break;
      case BLING_TEXN_CHECKER:
      case BLING_TEXN_GRAPH_PAPER: want = "SS-"; break;
      case BLING_TEXN_GRADIENT: want = "--F"; break;
      case BLING_TEXN_SCALE: want = "F--"; break;
      default: break;
    }
    const int ch[3] = {t.a, t.b, t.c};
    for (int k = 0; k < 3; k++) {
      if (want[k] == '-') continue;
      if (ch[k] < 0 || ch[k] >= i) return fail(i, "a child must be an earlier node");
      int ck = d.textures[ch[k]].kind;
      if (want[k] == 'S' ? !tex_is_spectrum(ck) : !tex_is_scalar(ck))
        return fail(i, "a child has the wrong value type");
      depth[i] = std::max(depth[i], depth[ch[k]] + 1);
    }
    if (depth[i] > BLING_TEX_MAX_DEPTH) return fail(i, "deeper than BLING_TEX_MAX_DEPTH");
    bool map2d = t.kind == BLING_TEXN_GRAPH_PAPER || t.kind == BLING_TEXN_IMAGE ||
                 t.kind == BLING_TEXN_CRYSTAL || t.kind == BLING_TEXN_IMAGE_SCALAR;
    bool map3d = t.kind == BLING_TEXN_PERLIN || t.kind == BLING_TEXN_FBM ||
                 t.kind == BLING_TEXN_CELL_NOISE;
    if (map2d && t.map_kind != BLING_MAP_UV && t.map_kind != BLING_MAP_PLANAR)
      return fail(i, "needs a uv or planar mapping");
    if (map3d && t.map_kind != BLING_MAP_IDENTITY3D) return fail(i, "needs an identity3d mapping");
    if ((t.kind == BLING_TEXN_FBM || t.kind == BLING_TEXN_CRYSTAL) &&
        (t.ivalue < 0 || t.ivalue > 64))
      return fail(i, "octaves out of 0..64");
    if (t.kind == BLING_TEXN_CELL_NOISE && (t.ivalue < BLING_DIST_EUCLIDIAN || t.ivalue > BLING_DIST_CHEBYSHEV))
      return fail(i, "unknown distance function");
    if (t.kind == BLING_TEXN_GRADIENT && (t.ivalue < 1 || !t.data))
      return fail(i, "a gradient needs steps");
    if ((t.kind == BLING_TEXN_IMAGE || t.kind == BLING_TEXN_IMAGE_SCALAR) &&
        (t.width <= 0 || t.height <= 0 || !t.pixels))
      return fail(i, "an image needs pixels");
  }
  for (int i = 0; i < d.n_materials; i++) {
    const bling_material& m = d.materials[i];
    for (int s = 0; s < 9; s++) {
      int r = s < 8 ? m.tex[s] : m.bump;
      if (r == 0) continue;
      bool ok = r >= 1 && r <= d.n_textures;
      if (ok) ok = s < 5 ? tex_is_spectrum(d.textures[r - 1].kind) : tex_is_scalar(d.textures[r - 1].kind);
      if (!ok) {
        snprintf(buf, sizeof buf, "material %d: %s %d names no %s texture node", i,
                 s < 8 ? "slot" : "bump", s, s < 5 ? "spectrum" : "scalar");
        err = buf;
        return false;
      }
    }
  }
  return true;
}

int bling_scene_create(bling_ctx* c, const bling_scene_desc* d, bling_scene** out) {
  if (!c || !d || !out) return BLING_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  *out = nullptr;
  if (!c->stream) return set_err(c, BLING_ERR_STATE, "context has no device");
  CK(c, cudaSetDevice(c->device));
  auto t0 = std::chrono::steady_clock::now();
  // ---- validate (mkTriangleMesh checks, TriangleMesh.hs:48-55)
  if (d->n_meshes < 0 || d->n_shapes < 0 || d->n_materials < 0 || d->n_lights < 0)
    return set_err(c, BLING_ERR_INVALID_ARG, "negative counts");
  if (d->n_materials > 0 && !d->materials)
    return set_err(c, BLING_ERR_INVALID_ARG, "null material array");
  if (d->n_lights > 0 && !d->lights) return set_err(c, BLING_ERR_INVALID_ARG, "null light array");
  for (int i = 0; i < d->n_lights; i++)
    if (d->lights[i].kind < BLING_LIGHT_DIRECTIONAL || d->lights[i].kind > BLING_LIGHT_SUNSKY)
      return set_err(c, BLING_ERR_INVALID_ARG, "light %d: unknown kind %d", i, d->lights[i].kind);
  for (int i = 0; i < d->n_materials; i++)
    if (d->materials[i].kind < BLING_MAT_MATTE || d->materials[i].kind > BLING_MAT_BLACKBODY ||
        (d->materials[i].kd_texture != BLING_TEX_CONSTANT &&
         !((d->materials[i].kd_texture == BLING_TEX_CHECKER ||
            d->materials[i].kd_texture == BLING_TEX_GRAPH_PAPER) &&
           (d->materials[i].kind == BLING_MAT_MATTE || d->materials[i].kind == BLING_MAT_PLASTIC ||
            d->materials[i].kind == BLING_MAT_SUBSTRATE))))
      return set_err(c, BLING_ERR_INVALID_ARG, "material %d: unknown kind %d", i,
                     d->materials[i].kind);
  {
    std::string terr;
    if (!check_textures(*d, terr)) return set_err(c, BLING_ERR_INVALID_ARG, "%s", terr.c_str());
  }
  for (int i = 0; i < d->n_meshes; i++) {
    const bling_mesh_desc& m = d->meshes[i];
    if (m.n_indices % 3 != 0)
      return set_err(c, BLING_ERR_INVALID_ARG, "mesh %d: number of indices must be multiple of 3", i);
    if (m.n_indices > 0 && (!m.indices || !m.vertices))
      return set_err(c, BLING_ERR_INVALID_ARG, "mesh %d: null arrays", i);
    for (int64_t k = 0; k < m.n_indices; k++) {
      if (m.indices[k] < 0) return set_err(c, BLING_ERR_INVALID_ARG, "mesh %d: contains negative indices", i);
      if (m.indices[k] >= m.n_vertices)
        return set_err(c, BLING_ERR_INVALID_ARG, "mesh %d: contains out of bounds indices", i);
    }
    if (m.material < 0 || m.material >= d->n_materials)
      return set_err(c, BLING_ERR_INVALID_ARG, "mesh %d: material %d out of range", i, m.material);
  }
  for (int i = 0; i < d->n_shapes; i++) {
    const bling_shape_desc& s = d->shapes[i];
    if (s.kind < BLING_SHAPE_SPHERE || s.kind > BLING_SHAPE_CYLINDER)
      return set_err(c, BLING_ERR_INVALID_ARG, "shape %d: unknown kind %d", i, s.kind);
    if (s.material < 0 || s.material >= d->n_materials)
      return set_err(c, BLING_ERR_INVALID_ARG, "shape %d: material %d out of range", i, s.material);
  }
  std::vector<int32_t> order;
  if (d->prim_order) {
    order.assign(d->prim_order, d->prim_order + d->n_meshes + d->n_shapes);
    std::vector<char> seen_m(d->n_meshes, 0), seen_s(d->n_shapes, 0);
    for (int32_t v : order) {
      if (v >= 0 ? v >= d->n_meshes : ~v >= d->n_shapes)
        return set_err(c, BLING_ERR_INVALID_ARG, "prim_order entry %d out of range", v);
      char& s = v >= 0 ? seen_m[v] : seen_s[~v];
      if (s) return set_err(c, BLING_ERR_INVALID_ARG, "prim_order entry %d repeated", v);
      s = 1;
    }
  } else {
    for (int i = 0; i < d->n_meshes; i++) order.push_back(i);
    for (int i = 0; i < d->n_shapes; i++) order.push_back(~i);
  }
  // ---- primitive list in primitive-ID order
  int64_t n_prims = 0;
  for (int32_t v : order) n_prims += v >= 0 ? d->meshes[v].n_indices / 3 : 1;
  if (n_prims == 0) return set_err(c, BLING_ERR_INVALID_ARG, "scene has no primitives");
  if (n_prims >= (int64_t(1) << 27)) return set_err(c, BLING_ERR_INVALID_ARG, "too many primitives");
  std::vector<float> lo(3 * n_prims), hi(3 * n_prims);
  // per primitive: kind/owner (mesh id or ~shape id) and triangle number
  std::vector<int32_t> prim_owner(n_prims), prim_tri(n_prims);
  {
    int64_t p = 0;
    for (int32_t v : order) {
      if (v >= 0) {
        const bling_mesh_desc& m = d->meshes[v];
        for (int64_t t = 0; t < m.n_indices / 3; t++, p++) {
          const float* a = m.vertices + 3 * m.indices[3 * t];
          const float* b = m.vertices + 3 * m.indices[3 * t + 1];
          const float* cc = m.vertices + 3 * m.indices[3 * t + 2];
          for (int k = 0; k < 3; k++) {
            lo[3 * p + k] = std::min(std::min(a[k], b[k]), cc[k]);
            hi[3 * p + k] = std::max(std::max(a[k], b[k]), cc[k]);
          }
          prim_owner[p] = v;
          prim_tri[p] = (int32_t)t;
        }
      } else {
        shape_world_bounds(d->shapes[~v], &lo[3 * p], &hi[3 * p]);
        prim_owner[p] = v;
        prim_tri[p] = 0;
        p++;
      }
    }
  }
  std::unique_ptr<bling_scene> S(new bling_scene());
  BvhBuildInput bi;
  bi.n = n_prims;
  bi.lo = lo.data();
  bi.hi = hi.data();
  bi.max_leaf = c->opts.bvh_leaf_size > 0 ? c->opts.bvh_leaf_size : 4;
  bi.wide = (c->opts.flags & BLING_FLAG_WIDE_BVH) != 0;
  bi.compact = (c->opts.flags & BLING_FLAG_COMPACT_BVH) != 0;
  BvhBuildOutput bo;
  // ---- BVH on the GPU (BLING_FLAG_GPU_BVH): boxes up, tree built in place
  GpuBvh gb;
  bool gpu_built = false;
  auto tb0 = std::chrono::steady_clock::now();  // the BVH construction alone
  if ((c->opts.flags & BLING_FLAG_GPU_BVH) && !bi.wide) {
    float *d_lo = nullptr, *d_hi = nullptr;
    int rc0 = upload(c, S->owned, lo.data(), lo.size(), &d_lo);
    if (!rc0) rc0 = upload(c, S->owned, hi.data(), hi.size(), &d_hi);
    if (rc0) return rc0;
    std::string berr;
    int brc = build_bvh_gpu(c->stream, d_lo, d_hi, n_prims, gb, berr);
    // the boxes were only needed for the build
    S->owned.erase(std::remove_if(S->owned.begin(), S->owned.end(),
                                  [&](void* p) { return p == d_lo || p == d_hi; }),
                   S->owned.end());
    cudaFree(d_lo);
    cudaFree(d_hi);
    if (brc) {
      gb.release();
      return set_err(c, brc == -2 ? BLING_ERR_OOM : BLING_ERR_CUDA, "%s", berr.c_str());
    }
    if (gb.depth < kBvhMaxDepth) {
      gpu_built = true;
    } else {
      gb.release();  // deeper than the traversal stack holds: build on the host
    }
  }
  if (!gpu_built && build_bvh(bi, bo) != 0)
    return set_err(c, BLING_ERR_INVALID_ARG, "BVH build failed (depth bound)");
  const double bvh_ms =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb0).count();
  // the wide layout when it was built (it is skipped for very deep trees)
  const bool wide = !gpu_built && bi.wide && bo.wide_depth >= 0;
  const bool compact = !gpu_built && !wide && bi.compact && bo.compact_ok;
  const std::vector<int32_t>& slot_prim = wide ? bo.slot_prim8 : (compact ? bo.slot_primC : bo.slot_prim);
  const std::vector<uint8_t>& slot_last = wide ? bo.slot_last8 : (compact ? bo.slot_lastC : bo.slot_last);
  // ---- leaf slots: in leaf order, or (GPU build) in primitive order, one per
  // leaf, gathered into leaf order on the device
  size_t n_slots = gpu_built ? (size_t)n_prims : slot_prim.size();
  std::vector<float> slots(12 * n_slots, 0.0f);
  for (size_t s = 0; s < n_slots; s++) {
    int32_t prim = gpu_built ? (int32_t)s : slot_prim[s];
    float* o = &slots[12 * s];
    int32_t flags = (gpu_built || slot_last[s]) ? SLOT_LAST : 0;
    int32_t v = prim_owner[prim];
    if (v >= 0) {
      const bling_mesh_desc& m = d->meshes[v];
      int64_t t = prim_tri[prim];
      const float* p1 = m.vertices + 3 * m.indices[3 * t];
      const float* p2 = m.vertices + 3 * m.indices[3 * t + 1];
      const float* p3 = m.vertices + 3 * m.indices[3 * t + 2];
      // e1 = p2 - p1, e2 = p3 - p1 (one binary32 subtraction each, as the reference)
      o[0] = p1[0];
      o[1] = p1[1];
      o[2] = p1[2];
      o[3] = p2[0] - p1[0];
      o[4] = p2[1] - p1[1];
      o[5] = p2[2] - p1[2];
      o[6] = p3[0] - p1[0];
      o[7] = p3[1] - p1[1];
      o[8] = p3[2] - p1[2];
    } else {
      int32_t si = ~v;
      memcpy(&o[0], &si, 4);
      flags |= SLOT_SHAPE;
    }
    memcpy(&o[9], &prim, 4);
    memcpy(&o[10], &flags, 4);
  }
  S->ctx = c;
  S->serial = ++g_scene_serial;
  for (int k = 0; k < 3; k++) {
    S->lo[k] = INFINITY;
    S->hi[k] = -INFINITY;
  }
  for (int64_t p = 0; p < n_prims; p++)
    for (int k = 0; k < 3; k++) {
      S->lo[k] = std::min(S->lo[k], lo[3 * p + k]);
      S->hi[k] = std::max(S->hi[k], hi[3 * p + k]);
    }
  int rc;
  if (gpu_built) {
    S->d_nodes = gb.nodes;  // owned by the scene from here on
    if (gb.nodes) S->owned.push_back(gb.nodes);
    gb.nodes = nullptr;
    float4* d_src = nullptr;
    if ((rc = upload(c, S->owned, (const float4*)slots.data(), slots.size() / 4, &d_src))) {
      gb.release();
      return rc;
    }
    float4* d_dst = nullptr;
    cudaError_t e = cudaMalloc(&d_dst, slots.size() * sizeof(float));
    if (e == cudaSuccess) {
      S->owned.push_back(d_dst);
      e = launch_gather_slots(d_src, gb.order, n_prims, d_dst, c->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    S->owned.erase(std::remove(S->owned.begin(), S->owned.end(), (void*)d_src), S->owned.end());
    cudaFree(d_src);
    gb.release();
    if (e != cudaSuccess)
      return set_err(c, e == cudaErrorMemoryAllocation ? BLING_ERR_OOM : BLING_ERR_CUDA,
                     "leaf slots: %s", cudaGetErrorString(e));
    S->d_slots = d_dst;
  } else if (wide) {
    if ((rc = upload(c, S->owned, (const uint4*)bo.nodes8.data(), bo.nodes8.size() / 4, &S->d_nodes8)))
      return rc;
  } else if (compact) {
    if ((rc = upload(c, S->owned, (const float4*)bo.nodesC.data(), bo.nodesC.size() / 4,
                     &S->d_nodesC)))
      return rc;
  } else {
    if ((rc = upload(c, S->owned, (const float4*)bo.nodes.data(), bo.nodes.size() / 4, &S->d_nodes)))
      return rc;
  }
  if (!gpu_built &&
      (rc = upload(c, S->owned, (const float4*)slots.data(), slots.size() / 4, &S->d_slots)))
    return rc;
  // ---- shapes on the device
  std::vector<DShape> shapes(d->n_shapes);
  std::vector<int32_t> shape_light(d->n_shapes, -1);
  {
    int32_t nl = d->n_lights;
    for (int32_t v : order)  // geometric lights follow the user lights, in primitive order
      if (v < 0 && d->shapes[~v].emissive) shape_light[~v] = nl++;
  }
  for (int i = 0; i < d->n_shapes; i++) {
    const bling_shape_desc& s = d->shapes[i];
    DShape& o = shapes[i];
    memset(&o, 0, sizeof o);
    o.kind = s.kind;
    o.material = s.material;
    o.light_id = shape_light[i];
    for (int k = 0; k < 6; k++) o.p[k] = s.params[k];
    memcpy(o.o2w, s.o2w, 64);
    memcpy(o.w2o, s.w2o, 64);
  }
  if ((rc = upload(c, S->owned, shapes.data(), shapes.size(), &S->d_shapes))) return rc;
  S->accel.nodes = S->d_nodes;
  S->accel.nodes8 = S->d_nodes8;
  S->accel.slots = S->d_slots;
  S->accel.shapes = S->d_shapes;
  S->accel.root_ref = gpu_built ? gb.root_ref : bo.root_ref;
  S->accel.root8 = bo.root8;
  S->accel.nodesC = S->d_nodesC;
  S->accel.rootC = bo.rootC;
  S->accel.wide = wide ? LAYOUT_WIDE : (compact ? LAYOUT_COMPACT : LAYOUT_BINARY);
  S->accel.n_shapes = d->n_shapes;
  S->accel.n_prims = n_prims;
  S->n_nodes = gpu_built ? gb.n_nodes
                         : (wide ? (int64_t)bo.nodes8.size() / 20
                                 : (compact ? (int64_t)bo.nodesC.size() / 8
                                            : (int64_t)bo.nodes.size() / 16));
  S->n_slots = (int64_t)n_slots;
  // ---- shading data for the path integrator
  if ((rc = integrator_upload_scene(c->stream, *d, order, prim_owner, prim_tri, shapes, shape_light,
                                    S->owned, S->shading, c->err)))
    return rc;
  CK(c, cudaStreamSynchronize(c->stream));
  auto t1 = std::chrono::steady_clock::now();
  S->stats.bvh_build_ms = bvh_ms;
  S->stats.nonfinite_pass = -1;
  S->stats.nonfinite_pixel[0] = S->stats.nonfinite_pixel[1] = S->stats.nonfinite_sample = -1;
  S->stats.scene_build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  S->stats.bvh_nodes = (uint64_t)S->n_nodes;
  S->stats.bvh_leaf_prims = (uint64_t)n_slots;
  size_t bytes = (gpu_built ? (size_t)gb.n_nodes * 16
                            : (wide ? bo.nodes8.size() : (compact ? bo.nodesC.size() : bo.nodes.size()))) *
                     4 +
                 slots.size() * 4 + shapes.size() * sizeof(DShape);
  S->stats.device_bytes = bytes + S->shading.bytes;
  *out = S.release();
  return BLING_OK;
}

void bling_scene_destroy(bling_scene* s) {
  if (!s) return;
  bling_ctx* c = s->ctx;
  {
    std::lock_guard<std::mutex> g(c->mu);
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (void* p : s->owned) cudaFree(p);
    s->owned.clear();
  }
  delete s;
}

int bling_scene_stats(bling_scene* s, bling_stats* out) {
  if (!s || !out) return BLING_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(s->ctx->mu);
  *out = s->stats;
  return BLING_OK;
}

int bling_trace_closest_device(bling_scene* s, const float* d_rays, size_t n, float* d_t,
                               int32_t* d_prim, float* d_b1b2) {
  if (!s || (n > 0 && (!d_rays || !d_t || !d_prim))) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = s->ctx;
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  CK(c, launch_trace_closest(s->accel, d_rays, (int64_t)n, d_t, d_prim, d_b1b2, c->d_counter,
                             c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  s->stats.rays_closest += n;
  return BLING_OK;
}

int bling_trace_any_device(bling_scene* s, const float* d_rays, size_t n, uint8_t* d_hit) {
  if (!s || (n > 0 && (!d_rays || !d_hit))) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = s->ctx;
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  CK(c, launch_trace_any(s->accel, d_rays, (int64_t)n, d_hit, c->d_counter, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  s->stats.rays_any += n;
  return BLING_OK;
}

int bling_trace_closest(bling_scene* s, const float* rays, size_t n, float* t, int32_t* prim,
                        float* b1b2) {
  if (!s || (n > 0 && (!rays || !t || !prim))) return BLING_ERR_INVALID_ARG;
  if (n == 0) return BLING_OK;
  bling_ctx* c = s->ctx;
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  QueryOut outs[3] = {{t, 4}, {prim, 4}, {b1b2, 8}};
  int rc = pipelined_query(c, rays, n, outs, b1b2 ? 3 : 2,
                           [&](const float* d_r, int64_t cn, void** d_out,
                               unsigned long long* d_counter, cudaStream_t ks) {
                             return launch_trace_closest(s->accel, d_r, cn, (float*)d_out[0],
                                                         (int32_t*)d_out[1],
                                                         b1b2 ? (float*)d_out[2] : nullptr,
                                                         d_counter, ks);
                           });
  if (rc) return rc;
  s->stats.rays_closest += n;
  return BLING_OK;
}

int bling_trace_any(bling_scene* s, const float* rays, size_t n, uint8_t* hit) {
  if (!s || (n > 0 && (!rays || !hit))) return BLING_ERR_INVALID_ARG;
  if (n == 0) return BLING_OK;
  bling_ctx* c = s->ctx;
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  QueryOut outs[1] = {{hit, 1}};
  int rc = pipelined_query(c, rays, n, outs, 1,
                           [&](const float* d_r, int64_t cn, void** d_out,
                               unsigned long long* d_counter, cudaStream_t ks) {
                             return launch_trace_any(s->accel, d_r, cn, (uint8_t*)d_out[0],
                                                     d_counter, ks);
                           });
  if (rc) return rc;
  s->stats.rays_any += n;
  return BLING_OK;
}

int bling_trace_counts(bling_scene* s, const float* rays, size_t n, uint64_t* nodes,
                       uint64_t* prims) {
  if (!s || !nodes || !prims || (n > 0 && !rays)) return BLING_ERR_INVALID_ARG;
  *nodes = *prims = 0;
  if (n == 0) return BLING_OK;
  bling_ctx* c = s->ctx;
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  size_t rb = 8 * n * sizeof(float);
  int rc = ensure_scratch(c, rb + 32);
  if (rc) return rc;
  float* d_r = (float*)c->d_scratch;
  unsigned long long* d_tot = (unsigned long long*)((char*)c->d_scratch + rb);
  CK(c, cudaMemcpyAsync(d_r, rays, rb, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaMemsetAsync(d_tot, 0, 16, c->stream));
  CK(c, launch_trace_counts(s->accel, d_r, (int64_t)n, d_tot, c->stream));
  unsigned long long tot[2];
  CK(c, cudaMemcpyAsync(tot, d_tot, 16, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  *nodes = tot[0];
  *prims = tot[1];
  return BLING_OK;
}

// ---------------------------------------------------------------- films
int bling_film_create_ex(bling_ctx* c, int32_t w, int32_t h, uint32_t flags, bling_film** out) {
  if (!c || !out || w <= 0 || h <= 0 || (int64_t)w * h > (int64_t(1) << 28) ||
      (flags & ~BLING_FILM_FP64))
    return BLING_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  *out = nullptr;
  CK(c, cudaSetDevice(c->device));
  std::unique_ptr<bling_film> f(new bling_film());
  f->ctx = c;
  f->width = w;
  f->height = h;
  size_t bytes = (size_t)w * h * 4 * sizeof(float);
  cudaError_t e = cudaMalloc(&f->d_film, bytes);
  if (e == cudaSuccess && (flags & BLING_FILM_FP64)) {
    e = cudaMalloc(&f->d_acc, 2 * bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(f->d_acc, 0, 2 * bytes, c->stream);
  }
  if (e != cudaSuccess) {
    cudaFree(f->d_film);
    return set_err(c, e == cudaErrorMemoryAllocation ? BLING_ERR_OOM : BLING_ERR_CUDA,
                   "film allocation: %s", cudaGetErrorString(e));
  }
  e = cudaMemsetAsync(f->d_film, 0, bytes, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    cudaFree(f->d_film);
    cudaFree(f->d_acc);
    return set_err(c, BLING_ERR_CUDA, "film clear: %s", cudaGetErrorString(e));
  }
  *out = f.release();
  return BLING_OK;
}

int bling_film_create(bling_ctx* c, int32_t w, int32_t h, bling_film** out) {
  return bling_film_create_ex(c, w, h, 0, out);
}

void bling_film_destroy(bling_film* f) {
  if (!f) return;
  {
    std::lock_guard<std::mutex> g(f->ctx->mu);
    cudaSetDevice(f->ctx->device);
    cudaStreamSynchronize(f->ctx->stream);
    cudaFree(f->d_film);
    cudaFree(f->d_acc);
    cudaFree(f->d_splat);
    cudaFree(f->d_sppm);
  }
  delete f;
}

int bling_film_fold(bling_film* f) {
  if (!f) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = f->ctx;
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  CK(c, film_fold(f, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return BLING_OK;
}

int bling_film_read_f64(bling_film* f, double* host) {
  if (!f || !host) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = f->ctx;
  if (!f->d_acc) return set_err(c, BLING_ERR_STATE, "film has no FP64 accumulator");
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  CK(c, film_fold(f, c->stream));
  CK(c, cudaMemcpyAsync(host, f->d_acc, (size_t)f->width * f->height * 4 * sizeof(double),
                        cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return BLING_OK;
}

int bling_film_clear(bling_film* f) {
  if (!f) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = f->ctx;
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  CK(c, cudaMemsetAsync(f->d_film, 0, (size_t)f->width * f->height * 16, c->stream));
  if (f->d_acc)
    CK(c, cudaMemsetAsync(f->d_acc, 0, (size_t)f->width * f->height * 32, c->stream));
  if (f->d_splat)
    CK(c, cudaMemsetAsync(f->d_splat, 0, (size_t)f->width * f->height * 12, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  cudaFree(f->d_sppm);  // the next SPPM pass starts from the initial radius again
  f->d_sppm = nullptr;
  f->sppm_pixels = 0;
  return BLING_OK;
}

int bling_film_read(bling_film* f, float* host) {
  if (!f || !host) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = f->ctx;
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  size_t n = (size_t)f->width * f->height * 4;
  if (f->d_acc) {
    // the FP64 totals, rounded once to float
    CK(c, film_fold(f, c->stream));
    std::vector<double> acc(n);
    CK(c, cudaMemcpyAsync(acc.data(), f->d_acc, n * sizeof(double), cudaMemcpyDeviceToHost,
                          c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < n; i++) host[i] = (float)acc[i];
    return BLING_OK;
  }
  CK(c, cudaMemcpyAsync(host, f->d_film, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return BLING_OK;
}

int bling_film_resolve(bling_film* f, float* host_rgb) {
  if (!f || !host_rgb) return BLING_ERR_INVALID_ARG;
  size_t np = (size_t)f->width * f->height;
  std::vector<float> px(4 * np);
  int rc = bling_film_read(f, px.data());
  if (rc) return rc;
  // getPixel with no splats (Image.hs:302-315), xyzToRgb (Spectrum.hs:162-168)
  for (size_t i = 0; i < np; i++) {
    float w = px[4 * i], x = px[4 * i + 1], y = px[4 * i + 2], z = px[4 * i + 3];
    float r = 0, gg = 0, b = 0;
    if (w != 0) {
      float wi = 1.0f / w;
      x = x * wi;
      y = y * wi;
      z = z * wi;
    } else {
      x = y = z = 0;
    }
    r = 3.240479f * x - 1.537150f * y - 0.498535f * z;
    gg = (-0.969256f) * x + 1.875991f * y + 0.041556f * z;
    b = 0.055648f * x - 0.204043f * y + 1.057311f * z;
    host_rgb[3 * i] = r;
    host_rgb[3 * i + 1] = gg;
    host_rgb[3 * i + 2] = b;
  }
  return BLING_OK;
}

int bling_film_read_splats(bling_film* f, float* host_xyz) {
  if (!f || !host_xyz) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = f->ctx;
  std::lock_guard<std::mutex> g(c->mu);
  size_t n = (size_t)f->width * f->height * 3;
  if (!f->d_splat) {  // no light pass yet: the reference's zeroed splat image
    std::fill(host_xyz, host_xyz + n, 0.0f);
    return BLING_OK;
  }
  CK(c, cudaSetDevice(c->device));
  CK(c, cudaMemcpyAsync(host_xyz, f->d_splat, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return BLING_OK;
}

int bling_film_resolve_splats(bling_film* f, float splat_weight, float* host_rgb) {
  if (!f || !host_rgb) return BLING_ERR_INVALID_ARG;
  size_t np = (size_t)f->width * f->height;
  std::vector<float> px(4 * np), sp(3 * np);
  int rc = bling_film_read(f, px.data());
  if (!rc) rc = bling_film_read_splats(f, sp.data());
  if (rc) return rc;
  // getPixel (Image.hs:302-315), xyzToRgb (Spectrum.hs:162-168)
  float sw = splat_weight;
  for (size_t i = 0; i < np; i++) {
    float w = px[4 * i], x = px[4 * i + 1], y = px[4 * i + 2], z = px[4 * i + 3];
    float sx = sp[3 * i], sy = sp[3 * i + 1], sz = sp[3 * i + 2];
    if (w == 0) {
      x = sw * sx;
      y = sw * sy;
      z = sw * sz;
    } else {
      float wi = 1.0f / w;
      x = sw * sx + x * wi;
      y = sw * sy + y * wi;
      z = sw * sz + z * wi;
    }
    host_rgb[3 * i] = 3.240479f * x - 1.537150f * y - 0.498535f * z;
    host_rgb[3 * i + 1] = (-0.969256f) * x + 1.875991f * y + 0.041556f * z;
    host_rgb[3 * i + 2] = 0.055648f * x - 0.204043f * y + 1.057311f * z;
  }
  return BLING_OK;
}

// ---------------------------------------------------------------- SPPM
namespace {
// the film's splat image, made on first use
int ensure_splats(bling_ctx* c, bling_film* f) {
  if (f->d_splat) return BLING_OK;
  size_t sbytes = (size_t)f->width * f->height * 3 * sizeof(float);
  cudaError_t e = cudaMalloc(&f->d_splat, sbytes);
  if (e != cudaSuccess) {
    f->d_splat = nullptr;
    return set_err(c, e == cudaErrorMemoryAllocation ? BLING_ERR_OOM : BLING_ERR_CUDA,
                   "splat image allocation: %s", cudaGetErrorString(e));
  }
  CK(c, cudaMemsetAsync(f->d_splat, 0, sbytes, c->stream));
  return BLING_OK;
}
// boundingSphere (AABB.hs:53-66) of the primitives' world bounds
void scene_sphere(const bling_scene* s, float wc[3], float& wr) {
  for (int k = 0; k < 3; k++) wc[k] = s->lo[k] + (s->hi[k] - s->lo[k]) * 0.5f;
  float e0 = s->hi[0] - wc[0], e1 = s->hi[1] - wc[1], e2 = s->hi[2] - wc[2];
  wr = sqrtf(e0 * e0 + e1 * e1 + e2 * e2);
}
}  // namespace

int bling_sppm_pass(bling_scene* s, bling_film* f, const bling_sppm_params* p, uint64_t pass) {
  if (!s || !f || !p) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = s->ctx;
  if (f->ctx != c) return set_err(c, BLING_ERR_INVALID_ARG, "film and scene belong to different contexts");
  if (p->photons < 0 || p->max_depth < 1 || p->max_depth > 24)
    return set_err(c, BLING_ERR_INVALID_ARG, "photons must be >= 0 and max_depth in 1..24");
  if (!(p->radius > 0) || !(p->alpha > 0 && p->alpha < 1))
    return set_err(c, BLING_ERR_INVALID_ARG, "radius must be > 0 and alpha in (0, 1)");
  SppmArgs a;
  memset(&a, 0, sizeof a);
  a.seed = p->seed;
  a.pass = pass;
  a.photons = p->photons;
  a.max_depth = p->max_depth;
  a.alpha = p->alpha;
  a.rp.width = f->width;
  a.rp.height = f->height;
  a.rp.strata_x = a.rp.strata_y = 1;  // mkRandomSampler 1 (SPPM.hs:150)
  a.rp.max_depth = p->max_depth;
  a.rp.rr_depth = 7;
  a.rp.filter_kind = p->filter_kind;
  memcpy(a.rp.filter_params, p->filter_params, sizeof a.rp.filter_params);
  a.rp.seed = p->seed;
  a.rp.sampler_kind = BLING_SAMPLER_RANDOM;
  int prc = check_render_params(c, &a.rp);
  if (prc) return prc;
  scene_sphere(s, a.wc, a.wr);
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  auto t0 = std::chrono::steady_clock::now();
  int rc = ensure_splats(c, f);
  if (rc) return rc;
  int64_t np = 0;
  rc = sppm_extent_pixels(a.rp, np, c->err);
  if (rc) return rc;
  if (!f->d_sppm || f->sppm_pixels != np) {  // first pass: every radius^2 = r * r, N = M = 0
    cudaFree(f->d_sppm);
    f->d_sppm = nullptr;
    f->sppm_pixels = 0;
    cudaError_t e = cudaMalloc(&f->d_sppm, (size_t)np * 12);
    if (e != cudaSuccess) {
      f->d_sppm = nullptr;
      return set_err(c, e == cudaErrorMemoryAllocation ? BLING_ERR_OOM : BLING_ERR_CUDA,
                     "SPPM statistics allocation: %s", cudaGetErrorString(e));
    }
    std::vector<float> r2(np, p->radius * p->radius);
    CK(c, cudaMemcpyAsync(f->d_sppm, r2.data(), (size_t)np * 4, cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemsetAsync((char*)f->d_sppm + (size_t)np * 4, 0, (size_t)np * 8, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    f->sppm_pixels = np;
  }
  SppmPixelStats px{(float*)f->d_sppm, (float*)f->d_sppm + np, (uint32_t*)((float*)f->d_sppm + 2 * np),
                    np};
  SppmResult res{};
  rc = sppm_pass(c->stream, s->accel, s->shading, a, f->d_film, f->d_splat, px, c->sp_ws, res,
                 c->err);
  if (rc) return rc;
  if (f->d_acc) {  // the camera samples' FP32 sums into the FP64 totals
    CK(c, film_fold(f, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
  }
  auto t1 = std::chrono::steady_clock::now();
  s->stats.last_pass_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  s->stats.rays_closest += res.rays_closest;
  s->stats.path_samples += res.camera_samples + res.photons;
  s->stats.nonfinite_drops += res.nonfinite;
  s->stats.degenerate_rays += res.degenerate;
  s->stats.light_splats += res.splats;
  return BLING_OK;
}

int bling_film_read_sppm_radii(bling_film* f, float* r2, int64_t capacity, int64_t* count) {
  if (!f || !count) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = f->ctx;
  std::lock_guard<std::mutex> g(c->mu);
  *count = f->d_sppm ? f->sppm_pixels : 0;
  if (!f->d_sppm || !r2) return BLING_OK;  // r2 = NULL asks for the count
  if (capacity < f->sppm_pixels)
    return set_err(c, BLING_ERR_BOUNDS, "radius buffer holds %lld of %lld pixels",
                   (long long)capacity, (long long)f->sppm_pixels);
  CK(c, cudaSetDevice(c->device));
  CK(c, cudaMemcpyAsync(r2, f->d_sppm, (size_t)f->sppm_pixels * 4, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return BLING_OK;
}

// ---------------------------------------------------------------- light tracer
int bling_light_pass(bling_scene* s, bling_film* f, const bling_light_params* p, uint64_t pass) {
  if (!s || !f || !p) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = s->ctx;
  if (f->ctx != c) return set_err(c, BLING_ERR_INVALID_ARG, "film and scene belong to different contexts");
  if (p->photons < 0 || p->max_depth < 0)
    return set_err(c, BLING_ERR_INVALID_ARG, "photons and max_depth must be >= 0");
  const bling_camera_desc& cam = s->shading.camera;
  if (!(cam.pixel_area > 0))
    return set_err(c, BLING_ERR_INVALID_ARG,
                   "the scene's camera has no world-to-raster transform and pixel area");
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  auto t0 = std::chrono::steady_clock::now();
  int src = ensure_splats(c, f);
  if (src) return src;
  LightPassArgs a;
  a.seed = p->seed;
  a.pass = pass;
  a.photons = p->photons;
  a.width = f->width;
  a.height = f->height;
  a.max_depth = p->max_depth;
  scene_sphere(s, a.wc, a.wr);
  LightPassResult res{};
  int rc = light_pass(c->stream, s->accel, s->shading, a, f->d_splat, c->lt_ws, res, c->err);
  if (rc) return rc;
  auto t1 = std::chrono::steady_clock::now();
  s->stats.last_pass_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  s->stats.rays_closest += res.rays_closest;
  s->stats.rays_any += res.rays_any;
  s->stats.path_samples += res.photons;
  s->stats.nonfinite_drops += res.nonfinite;
  s->stats.degenerate_rays += res.degenerate;
  s->stats.light_splats += res.splats;
  return BLING_OK;
}

// the latest render pass that dropped a sample, and that pass's first one
static void note_dropped(bling_scene* s, uint64_t pass, const PassResult& res) {
  if (res.nf_x < 0) return;
  s->stats.nonfinite_pass = (int64_t)pass;
  s->stats.nonfinite_pixel[0] = res.nf_x;
  s->stats.nonfinite_pixel[1] = res.nf_y;
  s->stats.nonfinite_sample = res.nf_n;
}

int bling_render_pass(bling_scene* s, bling_film* f, const bling_render_params* p, uint64_t pass) {
  return bling_render_pass_camera(s, f, p, nullptr, pass);
}

int bling_render_pass_camera(bling_scene* s, bling_film* f, const bling_render_params* p,
                             const bling_camera_desc* camera, uint64_t pass) {
  if (!s || !f || !p) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = s->ctx;
  if (f->ctx != c) return set_err(c, BLING_ERR_INVALID_ARG, "film and scene belong to different contexts");
  if (p->width != f->width || p->height != f->height)
    return set_err(c, BLING_ERR_INVALID_ARG, "render size %dx%d does not match film %dx%d", p->width,
                   p->height, f->width, f->height);
  int prc = check_render_params(c, p);
  if (prc) return prc;
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  PassResult res{};
  auto t0 = std::chrono::steady_clock::now();
  DevShading sh = s->shading;
  if (camera) sh.camera = *camera;
  const float box[6] = {s->lo[0], s->lo[1], s->lo[2], s->hi[0], s->hi[1], s->hi[2]};
  const bool bin = (c->opts.flags & BLING_FLAG_BIN_RAYS) != 0;
  int rc = integrator_render_pass(c->stream, s->accel, sh, *p, pass, f->d_film, f->width,
                                  f->height, c->ws, res, c->err, bin ? box : nullptr);
  if (rc) return rc;
  if (f->d_acc) {  // the pass's FP32 sums into the FP64 totals
    CK(c, film_fold(f, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
  }
  auto t1 = std::chrono::steady_clock::now();
  s->stats.last_pass_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  s->stats.rays_closest += res.rays_closest;
  s->stats.rays_any += res.rays_any;
  s->stats.path_samples += res.path_samples;
  s->stats.nonfinite_drops += res.nonfinite;
  s->stats.degenerate_rays += res.degenerate;
  note_dropped(s, pass, res);
  return BLING_OK;
}

// The no-allocation pass: the caller owns the film's device memory and the
// library's path state sits in a static device array (integrator.cu), so
// nothing here calls cudaMalloc/cudaFree.  See bling_gpu.h for the limits.
int bling_render_pass_noalloc(bling_scene* s, const bling_render_params* p, uint64_t pass,
                              float* d_film) {
  if (!s || !p || !d_film) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = s->ctx;
  int prc = check_render_params(c, p);
  if (prc) return prc;
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  PassResult res{};
  auto t0 = std::chrono::steady_clock::now();
  int rc = integrator_render_pass_noalloc(c->stream, s->accel, s->shading, *p, pass, d_film,
                                          p->width, p->height, res, c->err);
  if (rc) return rc;
  auto t1 = std::chrono::steady_clock::now();
  s->stats.last_pass_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  s->stats.rays_closest += res.rays_closest;
  s->stats.rays_any += res.rays_any;
  s->stats.path_samples += res.path_samples;
  s->stats.nonfinite_drops += res.nonfinite;
  s->stats.degenerate_rays += res.degenerate;
  note_dropped(s, pass, res);
  return BLING_OK;
}

// ---------------------------------------------------------------- batched jobs
int bling_batch_create(bling_ctx* c, const bling_batch_opts* o, bling_batch** out) {
  if (!c || !out) return BLING_ERR_INVALID_ARG;
  *out = nullptr;
  std::lock_guard<std::mutex> g(c->mu);
  if (!c->stream) return set_err(c, BLING_ERR_STATE, "context has no device");
  CK(c, cudaSetDevice(c->device));
  BatchConfig cfg;
  if (o) {
    if (o->slots) cfg.slots = o->slots;
    if (o->block_size) cfg.block = o->block_size;
    if (o->max_jobs) cfg.max_jobs = o->max_jobs;
    cfg.sort_rays = o->sort_rays != 0;
    cfg.graph_mode = o->graph_mode;
    if (o->iters_per_launch) cfg.iters_per_launch = o->iters_per_launch;
    if (o->max_run_iterations < 0)
      return set_err(c, BLING_ERR_INVALID_ARG, "max_run_iterations must be >= 0");
    cfg.max_run_iterations = o->max_run_iterations;
  } else {
    cfg.graph_mode = BLING_BATCH_PLAIN_LAUNCHES;
  }
  BatchEngine* e = nullptr;
  int rc = batch_create(c->device, c->stream, cfg, &e, c->err);
  if (rc) return rc;
  bling_batch* b = new bling_batch();
  b->ctx = c;
  b->eng = e;
  *out = b;
  return BLING_OK;
}

void bling_batch_destroy(bling_batch* b) {
  if (!b) return;
  {
    std::lock_guard<std::mutex> g(b->ctx->mu);
    cudaSetDevice(b->ctx->device);
    batch_destroy(b->eng);
  }
  delete b;
}

int bling_batch_submit(bling_batch* b, bling_scene* s, bling_film* f, const bling_render_params* p,
                       const bling_camera_desc* camera, uint64_t pass, int64_t* job_id) {
  if (!b || !s || !f || !p || !job_id) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = b->ctx;
  if (s->ctx != c || f->ctx != c)
    return set_err(c, BLING_ERR_INVALID_ARG, "scene, film and batch belong to different contexts");
  if (p->width != f->width || p->height != f->height)
    return set_err(c, BLING_ERR_INVALID_ARG, "render size %dx%d does not match film %dx%d", p->width,
                   p->height, f->width, f->height);
  int rc = check_render_params(c, p);
  if (rc) return rc;
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  int idx = 0;
  rc = batch_scene(b->eng, s->serial, s->accel, s->shading, s->lo, s->hi, idx, c->err);
  if (rc) return rc;
  const bling_camera_desc& cam = camera ? *camera : s->shading.camera;
  return batch_submit(b->eng, idx, cam, f->d_film, f->width, f->height, *p, pass, *job_id, c->err);
}

int bling_batch_step(bling_batch* b, int32_t iterations) {
  if (!b) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = b->ctx;
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  return batch_step(b->eng, iterations, c->err);
}

int bling_batch_run(bling_batch* b) {
  if (!b) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = b->ctx;
  std::lock_guard<std::mutex> g(c->mu);
  CK(c, cudaSetDevice(c->device));
  return batch_run(b->eng, c->err);
}

int bling_batch_job_status(bling_batch* b, int64_t job_id, uint64_t* done, uint64_t* total) {
  if (!b || !done || !total) return BLING_ERR_INVALID_ARG;
  bling_ctx* c = b->ctx;
  std::lock_guard<std::mutex> g(c->mu);
  return batch_job_status(b->eng, job_id, *done, *total, c->err);
}

int bling_batch_stats_get(bling_batch* b, bling_batch_stats* out) {
  if (!b || !out) return BLING_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(b->ctx->mu);
  BatchStats st;
  batch_stats(b->eng, st);
  out->rays_closest = st.rays_closest;
  out->rays_any = st.rays_any;
  out->path_samples = st.path_samples;
  out->nonfinite_drops = st.nonfinite;
  out->degenerate_rays = st.degenerate;
  out->iterations = st.iterations;
  out->samples_submitted = st.samples_submitted;
  out->samples_started = st.samples_started;
  out->jobs_submitted = st.jobs_submitted;
  out->jobs_done = st.jobs_done;
  out->jobs_active = st.jobs_active;
  out->device_bytes = (uint64_t)st.device_bytes;
  return BLING_OK;
}

// ---------------------------------------------------------------- host helpers
int bling_bvh_selftest(const float* lo, const float* hi, int64_t n, int32_t max_leaf,
                       int64_t* stats) {
  if (!lo || !hi || n <= 0 || !stats) return BLING_ERR_INVALID_ARG;
  BvhBuildInput bi;
  bi.n = n;
  bi.lo = lo;
  bi.hi = hi;
  bi.max_leaf = max_leaf > 0 ? max_leaf : 4;
  bi.wide = true;
  bi.compact = true;
  BvhBuildOutput bo;
  if (build_bvh(bi, bo) != 0) return BLING_ERR_INVALID_ARG;
  if (!bo.compact_ok) return -50;  // the 32-byte layout must exist for every tree
  stats[0] = (int64_t)bo.nodes.size() / 16;
  stats[1] = bo.wide_depth >= 0 ? (int64_t)bo.nodes8.size() / 20 : 0;
  stats[2] = bo.max_depth;
  stats[3] = bo.wide_depth;
  stats[4] = bo.leaves;
  return validate_bvh(bi, bo);
}
void bling_sunsky_eval(const float east[3], const float sun_dir[3], float turbidity, float u,
                       float v, float out[BLING_BANDS]) {
  SkyModel m;
  skyInit(east, sun_dir, turbidity, m);
  skyEval(m, u, v, out);
}
void bling_rgb_to_spectrum(int32_t illum, float r, float g, float b, float out[BLING_BANDS]) {
  const uint32_t* t = illum ? BLING_RGB_ILLUM_BITS : BLING_RGB_REFL_BITS;
  auto B = [&](int which, int i) { return fbits(t[which * 16 + i]); };
  for (int i = 0; i < 16; i++) {
    float w = B(BLING_BASIS_WHITE, i), cy = B(BLING_BASIS_CYAN, i), m = B(BLING_BASIS_MAGENTA, i),
          y = B(BLING_BASIS_YELLOW, i), rr = B(BLING_BASIS_RED, i), gg = B(BLING_BASIS_GREEN, i),
          bb = B(BLING_BASIS_BLUE, i);
    float v;
    // rgbToSpectrum (Spectrum.hs:146-159), band by band
    if (r <= g && r <= b)
      v = w * r + (g <= b ? cy * (g - r) + bb * (b - g) : cy * (b - r) + gg * (g - b));
    else if (g <= r && g <= b)
      v = w * g + (r <= b ? m * (r - g) + bb * (b - r) : m * (b - g) + rr * (r - b));
    else
      v = w * b + (r <= b ? y * (r - b) + gg * (g - r) : y * (g - b) + rr * (r - g));
    out[i] = v;
  }
}

void bling_spectrum_to_xyz(const float s[BLING_BANDS], float xyz[3]) {
  float a = 0, b = 0, cc = 0;
  for (int i = 0; i < 16; i++) {
    a = a + fbits(BLING_CIE_X_BITS[i]) * s[i];
    b = b + fbits(BLING_CIE_Y_BITS[i]) * s[i];
    cc = cc + fbits(BLING_CIE_Z_BITS[i]) * s[i];
  }
  float ys = fbits(BLING_CIE_Y_SUM_BITS);
  xyz[0] = a / ys;
  xyz[1] = b / ys;
  xyz[2] = cc / ys;
}

}  // extern "C"
