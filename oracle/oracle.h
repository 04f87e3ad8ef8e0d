/* C API of the CPU oracle.  TEST INFRASTRUCTURE ONLY: the parity checker and
 * the timed host-core baseline for the GPU path-tracing core.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it. */
#ifndef BLING_ORACLE_H
#define BLING_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#include "../include/bling_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_scene orc_scene;

int orc_scene_create(const bling_scene_desc* desc, orc_scene** out);
void orc_scene_destroy(orc_scene* s);
int64_t orc_scene_prim_count(const orc_scene* s);

/* closest hit by brute force over all primitives in primitive-ID order
 * (the reference's `nearest'` fold, Primitive.hs:29-43); rays SoA as in
 * bling_trace_closest.  nthreads <= 0: all cores. */
void orc_trace_closest_brute(const orc_scene* s, const float* rays, size_t n, float* t,
                             int32_t* prim, float* b1b2, int nthreads);
void orc_trace_any_brute(const orc_scene* s, const float* rays, size_t n, uint8_t* hit,
                         int nthreads);
/* the same answers through a conservative BVH of the oracle's own (faster) */
void orc_trace_closest_bvh(const orc_scene* s, const float* rays, size_t n, float* t,
                           int32_t* prim, float* b1b2, int nthreads);
void orc_trace_any_bvh(const orc_scene* s, const float* rays, size_t n, uint8_t* hit,
                       int nthreads);

/* The reference's kd-tree (Primitive/KdTree.hs:81-246, restated in
 * kdtree.h) over the primitives' world bounds, built once per scene.
 * stats (8 entries): interior nodes, leaves, empty leaves, primitive
 * references in leaves, largest leaf, deepest leaf, sum of leaf depths, the
 * depth limit round(8 + 3 ln N). */
int orc_kdtree_build(orc_scene* s, int nthreads, int64_t* stats);
/* closest / any hit through the kd-tree with the reference's traversal
 * order (traverse / traverse', KdTree.hs:209-246); counts (2 entries, may be
 * NULL): nodes visited, primitive tests */
int orc_trace_closest_kd(orc_scene* s, const float* rays, size_t n, float* t, int32_t* prim,
                         float* b1b2, int nthreads, uint64_t* counts);
int orc_trace_any_kd(orc_scene* s, const float* rays, size_t n, uint8_t* hit, int nthreads,
                     uint64_t* counts);
/* on != 0: the renderers (orc_render_pass, orc_light_pass, orc_sppm_pass)
 * trace through the kd-tree instead of the oracle's BVH (built first if
 * needed) */
int orc_scene_use_kdtree(orc_scene* s, int on, int nthreads);

/* Full render pass over the film-padded sample extent, film (w,X,Y,Z)
 * accumulated in place (width*height*4 floats).  Restates prender/tile
 * (Rendering.hs:111-150) with the path integrator (Path.hs).  Only the rows
 * y in [row_begin, row_end) of the sample extent are rendered when
 * row_end > row_begin (for bounded CPU samples); returns the number of path
 * samples taken and the number of closest/any queries issued. */
int orc_render_pass(const orc_scene* s, const bling_render_params* p, uint64_t pass,
                    float* film_wxyz, int row_begin, int row_end, int nthreads,
                    uint64_t* path_samples, uint64_t* rays_closest, uint64_t* rays_any);

/* radiance of one camera sample: li as XYZ plus the raster position */
/* orc_render_pass over the whole image into a binary64 film (the tile and
 * film sums in double precision), for reference renders of many passes */
int orc_render_pass_f64(const orc_scene* s, const bling_render_params* p, uint64_t pass,
                        double* film, int nthreads, uint64_t* path_samples);
int orc_sample_li(const orc_scene* s, const bling_render_params* p, uint64_t pass, int px,
                  int py, int n, float* out_xyz, float* out_raster, float* out_spectrum);

/* Photons [first, first + count) of one light-tracer pass (oneRay/nextVertex,
 * Renderer/LightTracer.hs:46-110) splatted into splat_xyz (width*height*3
 * floats, accumulated in place; splatSample, Image.hs:201-221) through the
 * scene's camera (sampleCam, Camera.hs:90-100).  max_depth > 0 ends a photon
 * after that many vertices (the reference has no limit).  stats: closest and
 * any-hit queries, splats added, non-finite splats dropped. */
int orc_light_pass(const orc_scene* s, int32_t width, int32_t height, uint64_t seed, uint64_t pass,
                   int32_t max_depth, int64_t first, int64_t count, float* splat_xyz, int nthreads,
                   uint64_t stats[4]);

/* One SPPM pass (Renderer/SPPM.hs:410-480): camera samples of the Random
 * sampler added to film (w,X,Y,Z), hit points, spatial hash, photon splats
 * into splat_xyz and the per-pixel statistics r2/n/m (stat_count entries over
 * the sample extent, updated in place).  stats: closest-hit queries, hit
 * points, splats, non-finite splats dropped. */
int orc_sppm_pass(const orc_scene* s, const bling_sppm_params* params, int32_t width, int32_t height,
                  uint64_t pass, float* film_wxyz, float* splat_xyz, float* r2, float* n, uint32_t* m,
                  int64_t stat_count, int nthreads, uint64_t stats[4]);

/* restated helpers, for known-answer tests */
void orc_rgb_to_spectrum(int illum, float r, float g, float b, float out[16]);
/* texture node `node` of the scene at shading point p and surface (u, v):
 * 16 bands for spectrum nodes, out[0] for scalar ones */
int orc_texture_eval(const orc_scene* s, int node, const float p[3], float u, float v,
                     float out[16]);
/* mkSunSkyLight east sunDir turbidity evaluated at (u, v) */
void orc_sunsky_eval(const float east[3], const float sun_dir[3], float turbidity, float u,
                     float v, float out[16]);
void orc_spectrum_to_xyz(const float s[16], float xyz[3]);
void orc_xyz_to_rgb(const float xyz[3], float rgb[3]);
float orc_filter_eval(int kind, const float* params, float x, float y);
void orc_filter_table(int kind, const float* params, float out[256]);
void orc_random_floats(uint64_t seed, uint64_t pass, int px, int py, uint32_t n, uint32_t dim,
                       int count, float* out);
uint32_t orc_permute(uint32_t i, uint32_t l, uint32_t p);

/* Transform constructors (Transform.hs), each writes m and m^-1 (2 x 16 floats) */
void orc_xf_translate(float dx, float dy, float dz, float out[32]);
void orc_xf_scale(float sx, float sy, float sz, float out[32]);
void orc_xf_rotate(int axis, float deg, float out[32]);
void orc_xf_look_at(const float pos[3], const float look[3], const float up[3], float out[32]);
void orc_xf_perspective(float fov, float n, float f, float out[32]);
void orc_xf_concat(const float a[32], const float b[32], float out[32]);
/* mkPerspectiveCamera c2w lr fd fov sx sy (Camera.hs:136-148) */
void orc_camera_perspective(const float c2w[32], float lens_radius, float focal_distance,
                            float fov, float sx, float sy, bling_camera_desc* out);

#ifdef __cplusplus
}
#endif
#endif
