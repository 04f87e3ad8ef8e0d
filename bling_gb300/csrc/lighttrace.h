// The light tracer's host interface (lighttrace.cu): one pass of photons
// splatted through the scene's camera into a film's splat image.
#pragma once
#include <cstdint>
#include <string>

#include "integrator.h"

namespace bgpu {

struct LightPassArgs {
  uint64_t seed, pass;
  int64_t photons;
  int32_t width, height;  // the splat image
  int32_t max_depth;      // vertices per photon; 0: until Russian roulette ends it
  float wc[3], wr;        // bounding sphere of the scene's primitives
};

struct LightPassResult {
  uint64_t rays_closest, rays_any, photons, splats, nonfinite, degenerate;
};

// grow-only photon slots, queues and counters, owned by a context
struct LightWorkspace {
  size_t capacity = 0;  // photon slots
  void* buffer = nullptr;
};

int light_pass(cudaStream_t stream, const DevAccel& A, const DevShading& S, const LightPassArgs& a,
               float* d_splat, LightWorkspace& ws, LightPassResult& res, std::string& err);
void light_workspace_free(LightWorkspace& ws);

}  // namespace bgpu
