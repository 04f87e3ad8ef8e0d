// The C ABI's handle types (include/bling_gpu.h), shared by api.cu and the
// render server (server.cpp).
#pragma once
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bling_gpu.h"
#include "batch.h"
#include "integrator.h"
#include "internal.h"
#include "lighttrace.h"
#include "sppm.h"

struct bling_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;      // where work is enqueued
  cudaStream_t own_stream = nullptr;  // the context's own stream
  std::mutex mu;
  std::string err;
  bling_opts opts{};
  // grow-only staging buffers for host-buffer queries
  void* d_scratch = nullptr;
  size_t scratch_bytes = 0;
  // next-ray counter of the persistent traversal kernels (calls are serialised)
  unsigned long long* d_counter = nullptr;
  // copy streams and events of the chunked host-buffer queries (made on first use)
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  cudaStream_t compute2 = nullptr;  // every other chunk of a host-buffer query
  cudaEvent_t ev_start = nullptr;
  cudaEvent_t ev_in[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t ev_run[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t ev_out[3] = {nullptr, nullptr, nullptr};
  bgpu::IntegratorWorkspace ws;
  bgpu::LightWorkspace lt_ws;  // photon slots of the light tracer (made on first use)
  bgpu::SppmWorkspace sp_ws;   // hit points, hash and photon slots of SPPM (made on first use)
};

struct bling_scene {
  bling_ctx* ctx = nullptr;
  bgpu::DevAccel accel{};
  float4* d_nodes = nullptr;
  uint4* d_nodes8 = nullptr;
  float4* d_nodesC = nullptr;
  float4* d_slots = nullptr;
  bgpu::DShape* d_shapes = nullptr;
  bgpu::DevShading shading{};
  std::vector<void*> owned;  // other device allocations
  bling_stats stats{};
  int64_t n_nodes = 0, n_slots = 0;
  int32_t root_ref = 0;
  float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // world bounds of all primitives
  uint64_t serial = 0;  // unique per process (batches key their scene tables on it)
  // frees what a creation that failed part way had allocated (on the current
  // device); bling_scene_destroy empties `owned` first
  ~bling_scene() {
    for (void* p : owned) cudaFree(p);
  }
};

struct bling_film {
  bling_ctx* ctx = nullptr;
  int32_t width = 0, height = 0;
  float* d_film = nullptr;  // width*height*4: the samples added since the last fold
  double* d_acc = nullptr;  // BLING_FILM_FP64: width*height*4 totals of the folded passes
  float* d_splat = nullptr; // width*height*3 XYZ splats of light passes (made on first use)
  // SPPM pixel statistics of the sample extent: r2, N (floats), M (uint32), made by the first pass
  void* d_sppm = nullptr;
  int64_t sppm_pixels = 0;
};

struct bling_batch {
  bling_ctx* ctx = nullptr;
  bgpu::BatchEngine* eng = nullptr;
};

namespace bgpu {
// the checks bling_render_pass applies to a job's parameters; sets the
// context's message and returns a BLING_ERR_* on failure (api.cu)
int check_render_params(bling_ctx* c, const bling_render_params* p);
// the same checks without a context: the message goes to err
int validate_render_params(const bling_render_params* p, std::string& err);
}  // namespace bgpu
