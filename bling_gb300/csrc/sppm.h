// Stochastic progressive photon mapping (sppm.cu): one pass of camera hit
// points, a spatial hash over them and a photon pass that splats into the
// film's splat image.
#pragma once
#include <cstdint>
#include <string>

#include "integrator.h"

namespace bgpu {

struct SppmArgs {
  uint64_t seed, pass;
  int64_t photons;      // requested per pass (mkSPPM n); the pass traces ceil(sqrt n)^2
  int32_t max_depth;    // camera path vertices (mkSPPM md)
  float alpha;          // radius reduction (mkSPPM alpha)
  bling_render_params rp;  // the camera pass: film size, filter, seed
  float wc[3], wr;      // bounding sphere of the scene's primitives
};

struct SppmResult {
  uint64_t rays_closest, camera_samples, hitpoints, photons, splats, nonfinite, degenerate;
};

// per-pixel statistics of the sample extent (PixelStats, SPPM.hs:245-262):
// radius^2, accumulated photon count N, photons of the current pass M
struct SppmPixelStats {
  float* r2;
  float* n;
  uint32_t* m;
  int64_t count;
};

// grow-only device buffers of the SPPM passes, owned by a context
struct SppmWorkspace {
  void* cam = nullptr;      // camera-pass sample accumulators and node queues
  size_t cam_samples = 0, cam_nodes = 0;
  void* hp = nullptr;       // hit points
  size_t hp_cap = 0;
  void* buckets = nullptr;  // bucket counts, offsets, cursors, block sums
  size_t bucket_cap = 0;
  void* entries = nullptr;  // bucket entries: positions (float4), then hit-point indices
  size_t entry_cap = 0;
  void* photons = nullptr;  // photon slots
  size_t photon_cap = 0;
  unsigned long long* counters = nullptr;
};

// the sample extent's pixel count (windowPixels of imageWindow')
int sppm_extent_pixels(const bling_render_params& rp, int64_t& count, std::string& err);

int sppm_pass(cudaStream_t stream, const DevAccel& A, const DevShading& S, const SppmArgs& a,
              float* d_film, float* d_splat, const SppmPixelStats& px, SppmWorkspace& ws,
              SppmResult& res, std::string& err);
void sppm_workspace_free(SppmWorkspace& ws);

}  // namespace bgpu
