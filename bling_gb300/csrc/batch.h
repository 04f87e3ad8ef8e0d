// Batched job engine: one persistent wavefront over many render jobs.
//
// A job is one pass of the path integrator (the work of bling_render_pass)
// over one scene into one film.  The engine keeps a fixed pool of path slots;
// every iteration
//
//   k_iter_begin  hands free slots the next path samples of the submitted jobs
//                 (in submission order) and resets the iteration's queues
//   k_regen       camera rays of the newly started samples (path regeneration)
//   k_bin_*       optional: reorders the bounce rays by scene, direction
//                 octant and origin cell (Morton order) before tracing
//   k_trace       closest hits,  k_shade  one vertex of every live path,
//   k_trace_shadow / k_trace_mis  the vertex's shadow and MIS rays,
//   k_resolve     radiance, continuation; finished paths are splatted into
//                 their job's film and their slots freed
//   k_iter_end    flips the live queues (and ends the device-side loop)
//
// so the queues stay full while samples remain, across jobs of different
// scenes, resolutions, sample counts and depths.  Each slot carries its job,
// scene, sample index and depth; the traversal kernels walk each ray's own
// scene.  A sample's random numbers depend only on its job's seed and pass
// and its pixel and sample number, so a job renders the same image in any mix
// of jobs (up to the order of the film's float additions).
#pragma once
#include <string>
#include <vector>

#include "integrator.h"

namespace bgpu {

struct BatchConfig {
  int64_t slots = 1 << 21;   // path slots (the capacity of every queue)
  int block = 128;           // threads per block of every stage (64 or 128)
  int max_jobs = 1024;       // job table entries (power of two)
  bool sort_rays = false;    // Morton binning of each iteration's bounce rays
  int graph_mode = 1;        // 0 plain launches, 1 a CUDA graph per iteration,
                             // 2 a conditional (while) graph running many iterations
  int iters_per_launch = 16; // iterations per graph launch in mode 2
  int64_t max_run_iterations = 0;  // batch_run's bound on iterations; 0 = derived from the work
};

struct BatchStats {
  uint64_t rays_closest = 0, rays_any = 0, path_samples = 0, nonfinite = 0, degenerate = 0;
  uint64_t iterations = 0, samples_submitted = 0, samples_started = 0;
  int64_t jobs_submitted = 0, jobs_done = 0, jobs_active = 0;
  double device_bytes = 0;
};

struct BatchEngine;

int batch_create(int device, cudaStream_t stream, const BatchConfig& cfg, BatchEngine** out,
                 std::string& err);
void batch_destroy(BatchEngine* b);
// registers a scene (once per key: the scene's serial number, never reused
// within a process) and returns its table index
int batch_scene(BatchEngine* b, uint64_t key, const DevAccel& A, const DevShading& S,
                const float lo[3], const float hi[3], int& index, std::string& err);
// submits samples [first, first + count) of one pass (count 0: all from
// first on); the samples keep their pass indices, so slices of one pass
// submitted as separate jobs render the film the whole pass renders
int batch_submit(BatchEngine* b, int scene, const bling_camera_desc& cam, float* d_film, int fw,
                 int fh, const bling_render_params& p, uint64_t pass, int64_t& job_id,
                 std::string& err, uint64_t first = 0, uint64_t count = 0);
// runs `iterations` wavefront iterations (fewer if all work is done) and
// updates the jobs' progress
int batch_step(BatchEngine* b, int iterations, std::string& err);
// steps until every submitted job is complete; BLING_ERR_TIMEOUT once more
// than the iteration bound (cfg.max_run_iterations, or one derived from the
// submitted work) has run; the jobs stay in flight and a later step or run
// continues them
int batch_run(BatchEngine* b, std::string& err);
// drops every incomplete job and every path in flight (after a failed step,
// before the caller releases the jobs' films): waits for the stream, stops
// sample generation at the samples submitted so far and empties the live
// queues.  Dropped jobs read as retired.  Later submits run normally.
int batch_cancel(BatchEngine* b, std::string& err);
int batch_job_status(BatchEngine* b, int64_t job_id, uint64_t& done, uint64_t& total,
                     std::string& err);
void batch_stats(BatchEngine* b, BatchStats& out);
bool batch_uses_wide(BatchEngine* b);

}  // namespace bgpu
