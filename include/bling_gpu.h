/*
 * bling_gpu.h -- C ABI of the GB300 path-tracing core for bling.
 *
 * The reference renderer is Haskell; its drop-in point is the `Renderer`
 * class (src/lib/Graphics/Bling/Rendering.hs:77-78), whose sampler renderer
 * `prender` (Rendering.hs:111-140) runs the path integrator
 * (src/lib/Graphics/Bling/Integrator/Path.hs) over 16x16 tiles, one pass at a
 * time, and reports `PassDone` after each pass.  A `GpuPathRenderer` instance
 * on the Haskell side calls this library through `foreign import ccall`:
 * one `bling_render_pass` per pass, then `bling_film_read` for the image.
 *
 * Everything below `prender` -- kd-tree/BVH traversal, ray/triangle and
 * ray/shape intersection, BSDF and light sampling, film accumulation -- runs
 * on one GPU behind these entry points.  There is no CPU fallback: every call
 * that needs the GPU fails with BLING_ERR_CUDA when none is usable.
 *
 * Conventions
 *  - Return value: BLING_OK (0) or a negative BLING_ERR_*; the message is kept
 *    per context (`bling_last_error`).  Nothing aborts.
 *  - All host buffers are owned by the caller and only read/written during
 *    the call.  Device memory is owned by the library until *_destroy.
 *  - A context owns one CUDA stream; calls on one context are serialised by
 *    an internal mutex, so a context may be shared between threads.
 *  - Matrices are 4x4 float, row-major, in the reference's `Matrix` layout
 *    (src/lib/Graphics/Bling/Transform.hs:29-42); a transform is the pair
 *    (m, m^-1) as in `MkTransform` (Transform.hs:124-127).
 *  - Spectra are 16 float bands over 400-700 nm (Spectrum.hs:33-46).
 */
#ifndef BLING_GPU_H
#define BLING_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BLING_ABI_VERSION 5

#define BLING_OK 0
#define BLING_ERR_INVALID_ARG (-1)
#define BLING_ERR_OOM (-2)
#define BLING_ERR_CUDA (-3)
#define BLING_ERR_TIMEOUT (-4)
#define BLING_ERR_BOUNDS (-5)
#define BLING_ERR_STATE (-6)

#define BLING_BANDS 16

typedef struct bling_ctx bling_ctx;
typedef struct bling_scene bling_scene;
typedef struct bling_film bling_film;

/* bling_opts.flags */
#define BLING_FLAG_WIDE_BVH 1u /* 8-wide quantised BVH layout instead of the binary one */
#define BLING_FLAG_COMPACT_BVH 4u /* binary BVH in 32-byte quantised nodes (one 256-bit
                                     load per visit) instead of 64-byte float nodes */
#define BLING_FLAG_BIN_RAYS 8u /* path integrator: sort each bounce's rays after the
                                  camera's by direction octant and origin cell
                                  (Morton order) before tracing them */
#define BLING_FLAG_GPU_BVH 2u  /* build the BVH on the GPU (Morton order and PLOC
                                  clustering, binary layout, one primitive per
                                  leaf) instead of the host's binned SAH; not with
                                  BLING_FLAG_WIDE_BVH.  A tree deeper than the
                                  traversal's stack allows is rebuilt on the host. */

typedef struct bling_opts {
  int32_t device;        /* CUDA device ordinal */
  uint32_t flags;        /* BLING_FLAG_* */
  int32_t block_size;    /* traversal block size, 0 = default */
  int32_t bvh_leaf_size; /* max primitives per BVH leaf, 0 = default */
} bling_opts;

/* ---- scene description (flat; replaces the closure records of
 *      Primitive.hs:21-27 / Reflection.hs:42 that cannot cross an FFI) ---- */

/* Materials (src/lib/Graphics/Bling/Material.hs).  Each parameter is the
 * constant field below or, through bling_material.tex, a texture expression
 * (bling_texture) evaluated at every hit's shading geometry. */
enum {
  BLING_MAT_MATTE = 0,   /* mkMatte kd sigma            (Material.hs:32-41) */
  BLING_MAT_PLASTIC = 1, /* mkPlastic kd ks roughness   (Material.hs:76-87) */
  BLING_MAT_METAL = 2,   /* mkMetal eta k roughness     (Material.hs:89-96) */
  BLING_MAT_GLASS = 3,   /* glassMaterial ior kr kt     (Material.hs:56-66) */
  BLING_MAT_MIRROR = 4,  /* mirrorMaterial kr: kr in ks (Material.hs:68-72) */
  BLING_MAT_SHINY_METAL = 5, /* mkShinyMetal kr ks rough: kr in kd (Material.hs:98-109) */
  BLING_MAT_TRANS_MATTE = 6, /* translucentMatte kr kt ks: kr in kd, ks in sigma (Material.hs:43-53) */
  BLING_MAT_SUBSTRATE = 7,   /* mkSubstrate kd ks ka urough vrough depth: ka in kt, urough in
                                roughness, vrough in sigma, depth in ior (Material.hs:111-127) */
  BLING_MAT_BLACKBODY = 8    /* blackBodyMaterial: a BSDF without components (Reflection.hs:337-338) */
};

typedef struct bling_material {
  int32_t kind;
  float sigma;     /* matte: Oren-Nayar sigma, 0 = Lambertian */
  float roughness; /* plastic/metal: Blinn exponent is 1/roughness */
  float ior;       /* glass */
  float kd[BLING_BANDS];  /* matte/plastic diffuse */
  float ks[BLING_BANDS];  /* plastic specular, glass and mirror reflection */
  float kt[BLING_BANDS];  /* glass transmission */
  float eta[BLING_BANDS]; /* metal */
  float k[BLING_BANDS];   /* metal */
  /* the texture of kd (matte, plastic, substrate), picked per hit from the
   * shading point p:
   *  - BLING_TEX_CONSTANT: kd;
   *  - BLING_TEX_CHECKER, checkerBoard (sx sy sz) kd kd2 (Texture.hs:209-219),
   *    params sx sy sz: kd where floor (x sx) + floor (y sy) + floor (z sz)
   *    is even, kd2 where it is odd;
   *  - BLING_TEX_GRAPH_PAPER, graphPaper lw (planarMapping (vu, vv) (ou, ov))
   *    kd kd2 (Texture.hs:172-207), params lw vu vv ou ov: with u = p.vu + ou,
   *    v = p.vv + ov, kd2 (the lines) where the fraction of |u| or |v| is
   *    below lw/2 or above 1 - lw/2, kd (the paper) elsewhere */
  int32_t kd_texture;
  float kd_tex_params[9];
  float kd2[BLING_BANDS];
  /* Textured parameters: tex[slot] = 0 keeps the constant field, n + 1 takes
   * node n of bling_scene_desc.textures (a spectrum-valued node for the
   * spectrum slots, a scalar-valued one for the scalar slots).  The slots
   * follow the fields above: BLING_SLOT_KD .. BLING_SLOT_IOR.  A textured kd
   * replaces kd_texture. */
  int32_t tex[8];
  /* bumpMapped d material (Reflection.hs:344-377): bump = n + 1 makes the
   * scalar node n the displacement, 0 for none */
  int32_t bump;
  int32_t reserved_tex;
} bling_material;
enum { BLING_TEX_CONSTANT = 0, BLING_TEX_CHECKER = 1, BLING_TEX_GRAPH_PAPER = 2 };
enum {
  BLING_SLOT_KD = 0, BLING_SLOT_KS = 1, BLING_SLOT_KT = 2, BLING_SLOT_ETA = 3, BLING_SLOT_K = 4,
  BLING_SLOT_SIGMA = 5, BLING_SLOT_ROUGHNESS = 6, BLING_SLOT_IOR = 7
};

/* Texture expressions (Texture.hs; the grammar of MaterialParser.hs:120-240).
 * A scene's textures are one array of nodes.  A node names its children by
 * index; every child comes before its parent in the array (child index <
 * node index), and a tree is at most BLING_TEX_MAX_DEPTH nodes deep.  The
 * mappings read the shading geometry: uv (u, v of the surface), planar and
 * identity3d (the shading point p in world space). */
#define BLING_TEX_MAX_DEPTH 8
enum {
  /* spectrum-valued */
  BLING_TEXN_CONSTANT = 0,    /* constant spectrum */
  BLING_TEXN_BLEND = 1,       /* spectrumBlend a b c: c scalar (Texture.hs:134-145) */
  BLING_TEXN_CHECKER = 2,     /* checkerBoard (p[0] p[1] p[2]) a b (Texture.hs:209-219) */
  BLING_TEXN_GRAPH_PAPER = 3, /* graphPaper p[0] map a b (Texture.hs:187-207): a paper, b lines */
  BLING_TEXN_GRADIENT = 4,    /* gradient (mkGradient steps) c (Texture.hs:221-248): c scalar;
                                 ivalue steps of 17 floats (position, spectrum) in data */
  BLING_TEXN_IMAGE = 5,       /* imageTexture of an RGB image, map (Texture.hs:87-108,128-129):
                                 width x height pixels, r g b bytes per pixel, in pixels */
  /* scalar-valued */
  BLING_TEXN_SCALAR = 16,     /* constant p[0] */
  BLING_TEXN_SCALE = 17,      /* scaleTexture p[0] p[1] a: p[0] + p[1] * a (Texture.hs:178-179) */
  BLING_TEXN_PERLIN = 18,     /* noiseTexture (identityMapping3d map) (Texture.hs:340-413) */
  BLING_TEXN_FBM = 19,        /* fbm ivalue p[0] over identityMapping3d map (Texture.hs:328-337) */
  BLING_TEXN_CELL_NOISE = 20, /* cellNoise (BLING_DIST_ ivalue) (identityMapping3d map)
                                 (Texture.hs:250-300) */
  BLING_TEXN_CRYSTAL = 21,    /* quasiCrystal ivalue map (Texture.hs:302-326) */
  BLING_TEXN_IMAGE_SCALAR = 22 /* imageTexture of a grey image, map: one byte per pixel */
};
enum { BLING_MAP_UV = 0, BLING_MAP_PLANAR = 1, BLING_MAP_IDENTITY3D = 2 };
enum {
  BLING_DIST_EUCLIDIAN = 0, BLING_DIST_EUCLIDIAN2 = 1, BLING_DIST_MANHATTAN = 2,
  BLING_DIST_CHEBYSHEV = 3
};
typedef struct bling_texture {
  int32_t kind;             /* BLING_TEXN_* */
  int32_t a, b, c;          /* children, -1 where the kind has none */
  int32_t ivalue;           /* octaves (fbm, crystal), distance (cell noise), steps (gradient) */
  int32_t map_kind;         /* BLING_MAP_* of image, graph paper, crystal, noise nodes */
  float map[16];            /* uv (uvMapping): su sv ou ov; planar (planarMapping): vu(3)
                               vv(3) ou ov; identity3d (identityMapping3d): the world-to-texture
                               matrix, row-major */
  float p[4];               /* the kind's numbers (see the kinds) */
  float spectrum[BLING_BANDS]; /* constant */
  const float* data;        /* gradient steps */
  const uint8_t* pixels;    /* image pixels, rows top to bottom */
  int32_t width, height;    /* image size */
} bling_texture;

/* A triangle mesh (mkTriangleMesh, Primitive/TriangleMesh.hs:39-60).
 * Vertices and normals are already in world space (the reference applies
 * o2w once at build, TriangleMesh.hs:58-59).  Indices are validated like
 * the reference does (TriangleMesh.hs:48-55). */
typedef struct bling_mesh_desc {
  const float* vertices; /* 3 * n_vertices */
  int64_t n_vertices;
  const int32_t* indices; /* n_indices, a multiple of 3 */
  int64_t n_indices;
  const float* normals; /* optional shading normals, 3 * n_vertices, or NULL */
  const float* uvs;     /* optional 2 * n_vertices, or NULL (default uvs) */
  int32_t material;
  int32_t reserved;
} bling_mesh_desc;

/* Analytic shapes (Shape.hs:22-38) placed by mkGeom (Primitive/Geometry.hs:14-36). */
enum {
  BLING_SHAPE_SPHERE = 0,  /* params: radius */
  BLING_SHAPE_QUAD = 1,    /* params: sx, sy */
  BLING_SHAPE_BOX = 2,     /* params: pmin xyz, pmax xyz */
  BLING_SHAPE_DISK = 3,    /* params: height, radius, inner radius, phimax (radians) */
  BLING_SHAPE_CYLINDER = 4 /* params: radius, zmin, zmax, phimax (radians) */
};

typedef struct bling_shape_desc {
  int32_t kind;
  int32_t material;
  float params[6];
  float o2w[16];
  float w2o[16];
  int32_t emissive; /* nonzero: the shape is an area light (Light.hs:64-70) */
  float emission[BLING_BANDS];
} bling_shape_desc;

/* Non-geometric lights (Light.hs:31-45). */
enum {
  BLING_LIGHT_DIRECTIONAL = 0, /* mkDirectional spectrum dir */
  BLING_LIGHT_POINT = 1,       /* mkPointLight spectrum pos */
  BLING_LIGHT_INFINITE = 2,    /* mkInfiniteAreaLight map w2l */
  BLING_LIGHT_SUNSKY = 3       /* mkInfiniteAreaLight (mkSunSkyLight east sunDir turbidity) w2l
                                  (SunSky.hs:12-24): Perez's sky and the solar disc, evaluated
                                  at continuous directions; vec = sunDir */
};

typedef struct bling_light_desc {
  int32_t kind;
  float spectrum[BLING_BANDS]; /* directional/point radiance/intensity */
  float vec[3];                /* directional: normalised direction; point: position;
                                  sun/sky: the sun's direction */
  const float* env;            /* infinite: env_w * env_h * 16 floats, row v, column u */
  int32_t env_w, env_h;
  float w2l[16];               /* infinite, sun/sky: world-to-light */
  float l2w[16];               /* infinite, sun/sky: light-to-world */
  float east[3];               /* sun/sky: the east direction */
  float turbidity;             /* sun/sky: the sky's turbidity */
} bling_light_desc;

/* A projective camera (ProjectiveCamera, Camera.hs:23-31; mkProjective,
 * Camera.hs:108-135).  w2r and pixel_area are what sampleCam uses
 * (Camera.hs:95-100): the light tracer needs them, path tracing does not
 * (zero them when no light tracing is done). */
typedef struct bling_camera_desc {
  float c2w[16], c2w_inv[16];
  float r2c[16], r2c_inv[16];
  float lens_radius;
  float focal_distance;
  float w2r[16];    /* world to raster: (inverse c2w <> p) <> s2r */
  float pixel_area; /* pw * ph at the focal length tan (fov / 2) */
  float reserved;
} bling_camera_desc;

/* The scene.  Primitive IDs follow the list handed to mkKdTree
 * (Scene.hs:37-43): `prim_order` lists the meshes (v >= 0 -> mesh v, which
 * expands to its triangles in index order) and shapes (v < 0 -> shape ~v) in
 * that order; NULL means all meshes, then all shapes.  Lights follow
 * `mkScene`: the non-geometric lights, then the emissive shapes in primitive
 * order (Scene.hs:39,42). */
typedef struct bling_scene_desc {
  const bling_mesh_desc* meshes;
  int32_t n_meshes;
  const bling_shape_desc* shapes;
  int32_t n_shapes;
  const bling_material* materials;
  int32_t n_materials;
  const bling_light_desc* lights;
  int32_t n_lights;
  const int32_t* prim_order; /* n_meshes + n_shapes entries, or NULL */
  bling_camera_desc camera;
  const bling_texture* textures; /* the texture nodes materials refer to */
  int32_t n_textures;
  int32_t reserved_desc;
} bling_scene_desc;

/* Pixel filters (Filter.hs:12-21). */
enum {
  BLING_FILTER_BOX = 0,
  BLING_FILTER_GAUSS = 1,    /* params: w, h, alpha */
  BLING_FILTER_MITCHELL = 2, /* params: w, h, B, C */
  BLING_FILTER_SINC = 3,     /* params: w, h, tau */
  BLING_FILTER_TRIANGLE = 4  /* params: w, h */
};

/* Samplers (Sampling.hs:85-132). */
enum {
  BLING_SAMPLER_STRATIFIED = 0, /* Stratified nu nv: jittered strata, shuffled dimensions */
  BLING_SAMPLER_RANDOM = 1      /* Random spp: independent uniforms for every dimension */
};

/* One render job: `SamplerRenderer sampler (mkPathIntegrator md sd)`
 * (Rendering.hs:96-103, Sampling.hs:101-132, Path.hs:30-39).  With
 * BLING_SAMPLER_RANDOM, `mkRandomSampler spp` is strata_x = spp, strata_y = 1:
 * strata_x * strata_y samples per pixel per pass, none of them stratified. */
typedef struct bling_render_params {
  int32_t width, height;
  int32_t strata_x, strata_y; /* stratified nu x nv samples per pixel per pass */
  int32_t max_depth;          /* path maxDepth */
  int32_t sample_depth;       /* path sampleDepth (stratified dimensions) */
  int32_t rr_depth;           /* Russian roulette after this depth; reference: 7 */
  int32_t filter_kind;
  float filter_params[4];
  uint64_t seed;
  int32_t sampler_kind;       /* BLING_SAMPLER_*; 0 = stratified */
  int32_t reserved;           /* must be 0 */
} bling_render_params;

typedef struct bling_stats {
  uint64_t rays_closest;    /* closest-hit queries (camera, continuation, BSDF-MIS) */
  uint64_t rays_any;        /* any-hit queries (shadow) */
  uint64_t path_samples;    /* completed camera paths; light passes add their photons, SPPM
                               passes their camera samples and photons */
  uint64_t nonfinite_drops; /* NaN/Inf samples skipped by the film (Image.hs:253-256) */
  uint64_t degenerate_rays; /* rays with a NaN component, answered without traversal */
  double bvh_build_ms;       /* the BVH construction (host or GPU builder) */
  double last_pass_ms;
  uint64_t bvh_nodes;
  uint64_t bvh_leaf_prims;
  uint64_t device_bytes;
  uint64_t light_splats;    /* splats of light and SPPM passes added to the splat image */
  double scene_build_ms;    /* all of bling_scene_create: checks, BVH, uploads */
  /* The latest render pass (bling_render_pass, bling_render_pass_noalloc)
   * that dropped a NaN/Inf sample, -1 if none has, and that pass's first
   * dropped sample: its pixel and its sample number within the pixel (the
   * sample the oracle or a debugger can replay). */
  int64_t nonfinite_pass;
  int32_t nonfinite_pixel[2];
  int32_t nonfinite_sample;
  int32_t reserved_stats;
} bling_stats;

/* ---- context ---- */
int bling_ctx_create(bling_ctx** out, const bling_opts* opts);
/* Destroy every scene and film of a context before the context itself. */
void bling_ctx_destroy(bling_ctx* ctx);
const char* bling_last_error(bling_ctx* ctx);
/* Runs the context's work on an external CUDA stream (a cudaStream_t, e.g.
 * the caller's current stream) instead of its own; NULL restores the
 * context's own stream.  Calls still synchronise that stream before return. */
int bling_ctx_set_stream(bling_ctx* ctx, void* stream);
int bling_abi_version(void);

/* ---- scenes: copies the host arrays, builds and uploads the BVH ----
 * replaces mkScene/mkKdTree (Scene.hs:37-43, Primitive/KdTree.hs:107-112) */
int bling_scene_create(bling_ctx* ctx, const bling_scene_desc* desc, bling_scene** out);
void bling_scene_destroy(bling_scene* scene);

/* ---- ray queries over host buffers (SoA rays: ox oy oz dx dy dz tmin tmax,
 *      each n floats, i.e. rays[k*n + i]) ----
 * The rays go through the device in chunks: copied in and out on two copy
 * streams of the context and traced alternately on the context's stream and
 * a second compute stream of its own, all ordered after the work already
 * queued on the context's stream.  The call returns when every result is in
 * host memory.
 * bling_trace_closest replaces `scIntersect` (Scene.hs:49-51) on a batch:
 * the nearest hit, ties to the larger primitive ID as the reference's
 * `nearest'` fold does (Primitive.hs:29-43, TriangleMesh.hs:166).
 * prim[i] = -1 on a miss.  b1b2 may be NULL (2n floats: the barycentrics
 * of triangle hits, 0 for shapes).  A ray with a NaN component gets
 * prim[i] = -2 and t[i] = NaN without traversal (the reference's walk would
 * visit every node and report a NaN-distance hit); bling_trace_any reports
 * such rays as occluded, as triangleIntersects does for NaN. */
int bling_trace_closest(bling_scene* scene, const float* rays, size_t n, float* t,
                        int32_t* prim, float* b1b2);
/* replaces `occluded` (Scene.hs:45-47): hit[i] = 1 when any primitive is hit
 * within [tmin, tmax]. */
int bling_trace_any(bling_scene* scene, const float* rays, size_t n, uint8_t* hit);

/* Device-pointer variants: the same queries over buffers already resident on
 * the device (rays: 8*n floats SoA), launched on the context's stream and
 * synchronised before return. */
int bling_trace_closest_device(bling_scene* scene, const float* d_rays, size_t n, float* d_t,
                               int32_t* d_prim, float* d_b1b2);
int bling_trace_any_device(bling_scene* scene, const float* d_rays, size_t n, uint8_t* d_hit);

/* Work of the closest-hit traversal on a batch of host rays, as the
 * reference's dbgTraverse counts it (Primitive/KdTree.hs:252-281): BVH nodes
 * visited and leaf primitives tested, summed over the batch.  The walk is
 * depth-first with each leaf tested as soon as it is reached, as a CPU walk
 * of the same tree would go (the query kernels postpone leaves to keep a
 * warp's lanes together, which can visit a few more nodes). */
int bling_trace_counts(bling_scene* scene, const float* rays, size_t n, uint64_t* nodes_visited,
                       uint64_t* prims_tested);

/* ---- films and passes ---- */
int bling_film_create(bling_ctx* ctx, int32_t width, int32_t height, bling_film** out);
/* BLING_FILM_FP64: compensated accumulation for long renders (thousands of
 * samples per pixel).  Samples are added to an FP32 film by the kernels as
 * usual; after every bling_render_pass the pass's FP32 sums are added into
 * FP64 totals and the FP32 film is zeroed, so FP32 only ever sums one pass.
 * bling_film_read returns the totals rounded once to float;
 * bling_film_read_f64 returns them as doubles.  Batched jobs write the FP32
 * part; bling_film_fold folds it (reads fold too).  The reference film is
 * FP32 (Image.hs:39-82): its sums stay within its rounding. */
#define BLING_FILM_FP64 1u
int bling_film_create_ex(bling_ctx* ctx, int32_t width, int32_t height, uint32_t flags,
                         bling_film** out);
int bling_film_fold(bling_film* film);
int bling_film_read_f64(bling_film* film, double* host_wxyz);
void bling_film_destroy(bling_film* film);
int bling_film_clear(bling_film* film);
/* copies the (weight, X, Y, Z) film, width*height*4 floats (Image.hs:64-82) */
int bling_film_read(bling_film* film, float* host_wxyz);
/* resolves to linear sRGB floats, width*height*3 (getPixel/xyzToRgb,
 * Image.hs:302-315, Spectrum.hs:162-168) */
int bling_film_resolve(bling_film* film, float* host_rgb);

/* One pass of `prender` (Rendering.hs:127-138): every pixel of the
 * filter-padded sample extent gets strata_x*strata_y path samples, added to
 * the film.  `pass` selects the random stream (seed, pass). */
int bling_render_pass(bling_scene* scene, bling_film* film, const bling_render_params* params,
                      uint64_t pass);
/* The same pass through another camera (NULL: the scene's), for an image
 * size the scene's camera was not built for (the reference builds the camera
 * for the image size, Camera.hs:108-147). */
int bling_render_pass_camera(bling_scene* scene, bling_film* film,
                             const bling_render_params* params, const bling_camera_desc* camera,
                             uint64_t pass);

int bling_scene_stats(bling_scene* scene, bling_stats* out);

/* ---- stochastic progressive photon mapping ----
 * replaces the reference's SPPM renderer (Renderer/SPPM.hs:410-480).  One
 * pass: one Random-sampler camera sample per pixel of the sample extent
 * records hit points at non-specular surfaces (following specular
 * reflection and transmission both) and adds the emission it sees to the
 * film; a spatial hash over the hit points; ceil(sqrt photons)^2 photons
 * splat hpF * f * li / (|wi.ng| r^2 pi) into the splat image for every hit
 * point within its radius; each pixel's radius shrinks by alpha
 * (statsUpdate).  The film keeps the per-pixel radii between passes
 * (bling_film_clear resets them).  After n passes the reference's splat
 * weight is 1 / (n * ceil(sqrt photons)^2) (SPPM.hs:460). */
typedef struct bling_sppm_params {
  int64_t photons;        /* photons per pass (mkSPPM n) */
  int32_t max_depth;      /* camera path vertices (mkSPPM md), 1..24 */
  float radius;           /* initial search radius (mkSPPM r) */
  float alpha;            /* radius reduction (mkSPPM alpha), in (0, 1) */
  int32_t filter_kind;    /* the job's pixel filter, for the camera samples */
  float filter_params[4];
  uint64_t seed;
} bling_sppm_params;
int bling_sppm_pass(bling_scene* scene, bling_film* film, const bling_sppm_params* params,
                    uint64_t pass);
/* copies the per-pixel squared radii of the sample extent (row-major over
 * imageWindow', Image.hs:170-176) into r2 (capacity floats); *count gets the
 * number of pixels, 0 before the first SPPM pass.  r2 = NULL only asks for
 * the count. */
int bling_film_read_sppm_radii(bling_film* film, float* r2, int64_t capacity, int64_t* count);

/* ---- light tracer ----
 * replaces the reference's LightTracer renderer (Renderer/LightTracer.hs:
 * 20-110): photons leave the lights (sampleLightRay, Scene.hs:121-135), bounce
 * by adjoint BSDF sampling and connect every vertex to the camera
 * (connectCam, sampleCam: Camera.hs:90-100); unoccluded connections are added
 * to the film's splat image (splatSample, Image.hs:201-221).  The scene's
 * camera must carry w2r and pixel_area (mkProjective, Camera.hs:108-147). */
typedef struct bling_light_params {
  int64_t photons;   /* photons per pass (mkLightTracer ppp) */
  uint64_t seed;     /* with the pass index, selects the random stream */
  int32_t max_depth; /* vertices per photon; 0 = until Russian roulette ends it (the reference) */
  int32_t reserved;
} bling_light_params;
int bling_light_pass(bling_scene* scene, bling_film* film, const bling_light_params* params,
                     uint64_t pass);
/* copies the splat image, width*height*3 floats (X, Y, Z); zeros before the
 * first light pass.  bling_film_clear clears it too. */
int bling_film_read_splats(bling_film* film, float* host_xyz);
/* getPixel with splat weight sw (Image.hs:302-315): the film's weighted mean
 * plus sw times the splats, to linear sRGB floats, width*height*3.  After n
 * light passes of ppp photons the reference's sw is 1 / (n * ppp)
 * (LightTracer.hs:44). */
int bling_film_resolve_splats(bling_film* film, float splat_weight, float* host_rgb);

/* One render pass, like bling_render_pass, that allocates no device memory.
 * No counterpart in the reference: it serves callers that cannot call
 * cudaMalloc while rendering -- for instance a render server whose device
 * memory is reserved up front for resident scenes and films (a fixed HBM
 * budget), or a host that shares the GPU with another caching allocator --
 * where an allocation in the middle of a frame could fail for lack of memory,
 * and cudaMalloc/cudaFree would stall work on the device.
 *
 *  - The film is the caller's device buffer `d_film_wxyz`, width*height*4
 *    floats (w, X, Y, Z), accumulated in place (zero it before the first pass).
 *    It must be device (or managed) memory of the scene's device: anything
 *    else is refused with BLING_ERR_INVALID_ARG before any launch.
 *  - The path state lives in a static device array inside the library,
 *    reserved in every process that loads it on every GPU it runs on (about
 *    35 MiB), so one call renders at most 65536 path samples: sample-extent
 *    pixels x strata_x x strata_y.  Larger passes return BLING_ERR_BOUNDS
 *    with the sizes in the message; split the image or use bling_render_pass.
 *  - The first call on a device looks up that array's device address (set-up,
 *    once per device); make that first call before any stream capture.
 *  - All calls share the array.  Calls whose work overlaps on the GPU -- on
 *    different contexts or streams of one device -- race on it and must be
 *    serialised by the caller; calls on one context already are.
 *  - Counters, statistics and errors are as for bling_render_pass. */
int bling_render_pass_noalloc(bling_scene* scene, const bling_render_params* params, uint64_t pass,
                              float* d_film_wxyz);

/* ---- batched jobs: one persistent wavefront over many render jobs ----
 * No counterpart in the reference, whose renderer runs one job at a time
 * (Renderer.render, Rendering.hs:77-78).  A job is one bling_render_pass of a
 * scene into a film; a batch keeps a fixed pool of path slots that started
 * paths never leave until they end, and hands free slots the next samples of
 * the submitted jobs in submission order (path regeneration), so the ray
 * queues stay full across jobs of different scenes, sizes, sample counts and
 * depths.  A job's film gets the same samples, with the same random numbers,
 * as bling_render_pass(scene, film, params, pass) would add, up to the order
 * of the float additions into the film.
 *
 *  - Scenes and films must belong to the batch's context, and all scenes of a
 *    batch must share the BVH layout (BLING_FLAG_WIDE_BVH); they must outlive
 *    the batch's use of them.  A film must not be read, cleared or rendered
 *    by other calls while a job writes it.
 *  - bling_batch_submit only enqueues; bling_batch_step runs `iterations`
 *    wavefront iterations (each advances every live path by one bounce and
 *    starts new paths in free slots) and synchronises; bling_batch_run steps
 *    until every submitted job is complete.
 *  - Jobs may be submitted between steps while others are in flight
 *    (continuous batching).  The job table holds max_jobs incomplete jobs;
 *    a submit beyond that returns BLING_ERR_STATE. */
typedef struct bling_batch bling_batch;

#define BLING_BATCH_PLAIN_LAUNCHES 0 /* each iteration's kernels launched one by one */
#define BLING_BATCH_GRAPH 1          /* each iteration replayed from one CUDA graph */
#define BLING_BATCH_DEVICE_LOOP 2    /* a conditional (while) graph runs up to
                                        iters_per_launch iterations per launch and
                                        stops early when no work is left */

typedef struct bling_batch_opts {
  int64_t slots;            /* path slots, the capacity of every queue; 0 = 2^21 */
  int32_t block_size;       /* threads per block, 64 or 128; 0 = 128 */
  int32_t max_jobs;         /* job table entries, a power of two; 0 = 1024 */
  int32_t sort_rays;        /* 1: bin each iteration's bounce rays by scene, direction
                               octant and origin cell (Morton order) before tracing */
  int32_t graph_mode;       /* BLING_BATCH_* ; default (0 given) is plain launches */
  int32_t iters_per_launch; /* BLING_BATCH_DEVICE_LOOP only; 0 = 16 */
  int32_t max_run_iterations; /* bling_batch_run returns BLING_ERR_TIMEOUT after this many
                                 iterations with jobs still incomplete (they stay in flight);
                                 0 = a bound derived from the submitted work */
} bling_batch_opts;

typedef struct bling_batch_stats {
  uint64_t rays_closest, rays_any, path_samples, nonfinite_drops, degenerate_rays;
  uint64_t iterations, samples_submitted, samples_started;
  int64_t jobs_submitted, jobs_done, jobs_active;
  uint64_t device_bytes;
} bling_batch_stats;

int bling_batch_create(bling_ctx* ctx, const bling_batch_opts* opts, bling_batch** out);
void bling_batch_destroy(bling_batch* batch);
/* camera: NULL renders through the scene's camera; a job at another image
 * size than the scene's camera was made for passes its own camera (the
 * reference builds the camera for the image size, Camera.hs:108-147) */
int bling_batch_submit(bling_batch* batch, bling_scene* scene, bling_film* film,
                       const bling_render_params* params, const bling_camera_desc* camera,
                       uint64_t pass, int64_t* job_id);
int bling_batch_step(bling_batch* batch, int32_t iterations);
int bling_batch_run(bling_batch* batch);
/* samples finished and submitted of a job; done == total once it is complete */
int bling_batch_job_status(bling_batch* batch, int64_t job_id, uint64_t* samples_done,
                           uint64_t* samples_total);
int bling_batch_stats_get(bling_batch* batch, bling_batch_stats* out);

/* ---- render server: continuous batching of render jobs ----
 * No counterpart in the reference.  Scenes stay resident (their BVHs in
 * device memory); callers on any thread submit jobs, each one pass of a
 * scene at its own size, sample count, depth and camera.  A worker thread
 * admits jobs in arrival order while the device memory budget -- the
 * batch's path state plus 16 bytes per pixel of every admitted job's film --
 * and the job table allow, merges their samples into one shared wavefront
 * (a bling_batch) and runs it `iters_per_step` iterations at a time; jobs
 * arriving meanwhile join at the next step.  A finished film is copied to
 * the host and its device memory released; bling_server_wait hands it over.
 * Each job's film is the one bling_render_pass would produce for it, up to
 * the order of the float additions.  Scenes must outlive their jobs.  The
 * server uses the context's stream of the moment it was created. */
typedef struct bling_server bling_server;

typedef struct bling_server_opts {
  bling_batch_opts batch;    /* the shared wavefront; graph_mode 0 selects BLING_BATCH_GRAPH */
  uint64_t hbm_budget_bytes; /* path state + films of admitted jobs; 0 = 40 GiB */
  int32_t iters_per_step;    /* wavefront iterations between admission rounds; 0 = 4 */
  int32_t reserved;
} bling_server_opts;

typedef struct bling_job_times {
  double submitted, admitted, finished; /* seconds since the server was created */
  uint64_t samples;                     /* path samples of the job */
} bling_job_times;

typedef struct bling_server_stats {
  int64_t jobs_submitted, jobs_admitted, jobs_done, jobs_failed, jobs_running, jobs_pending;
  uint64_t samples_done, rays_closest, rays_any, iterations;
  uint64_t budget_bytes, bytes_in_use, peak_bytes_in_use;
} bling_server_stats;

int bling_server_create(bling_ctx* ctx, const bling_server_opts* opts, bling_server** out);
/* finishes the admitted jobs; pending ones fail with BLING_ERR_STATE */
void bling_server_destroy(bling_server* server);
/* thread-safe; camera NULL = the scene's camera.  A job whose film alone
 * exceeds the budget is refused with BLING_ERR_BOUNDS. */
int bling_server_submit(bling_server* server, bling_scene* scene, const bling_render_params* params,
                        const bling_camera_desc* camera, uint64_t pass, int64_t* ticket);
/* blocks until the job is done (timeout_ms < 0: no limit; BLING_ERR_TIMEOUT
 * otherwise), copies its (w, X, Y, Z) film to host_wxyz (width*height*4
 * floats, may be NULL) and its timestamps to times (may be NULL), and
 * forgets the ticket.  A failed job returns its error code. */
int bling_server_wait(bling_server* server, int64_t ticket, int32_t timeout_ms, float* host_wxyz,
                      bling_job_times* times);
int bling_server_stats_get(bling_server* server, bling_server_stats* out);
const char* bling_server_last_error(bling_server* server);
/* Test hook (no counterpart in the reference): after `after_steps` more
 * wavefront steps, the next step fails on the host with BLING_ERR_CUDA
 * without launching anything, as a failed launch would; -1 disarms.  The
 * running jobs fail, the batch drops their work before their films are
 * released, and later jobs render normally. */
int bling_server_debug_fail_step(bling_server* server, int32_t after_steps);

/* ---- host helpers for building scenes (no GPU needed) ---- */
/* Builds the BVH of n primitive boxes (lo/hi: 3n floats each) on the host and
 * checks its structure: each primitive in exactly one leaf, every stored box
 * (binary, quantised 8-wide and 32-byte quantised binary) containing its
 * subtree.  stats (5 entries):
 * binary inner nodes, wide nodes (0 when the wide layout was skipped), binary
 * depth, wide depth, leaves.  Returns 0 or a negative code of the first
 * violation.  The replacement of mkKdTree (Primitive/KdTree.hs:107-112) as a
 * testable unit. */
int bling_bvh_selftest(const float* lo, const float* hi, int64_t n, int32_t max_leaf,
                       int64_t* stats);
/* The sun/sky map of mkSunSkyLight east sunDir turbidity at (u, v)
 * (SunSky.hs:12-24), computed on the host.  BLING_LIGHT_SUNSKY lights
 * evaluate the same expression on the device, where sinf/cosf/acosf/expf/
 * powf may round differently in the last bit. */
void bling_sunsky_eval(const float east[3], const float sun_dir[3], float turbidity, float u,
                       float v, float out[BLING_BANDS]);
/* rgbToSpectrumRefl / rgbToSpectrumIllum (Spectrum.hs:140-159) */
void bling_rgb_to_spectrum(int32_t illuminant, float r, float g, float b, float out[BLING_BANDS]);
/* spectrumToXYZ (Spectrum.hs:349-355) */
void bling_spectrum_to_xyz(const float s[BLING_BANDS], float xyz[3]);

#ifdef __cplusplus
}
#endif
#endif /* BLING_GPU_H */
