"""ctypes mirrors of the C ABI structs declared in include/bling_gpu.h.

The same layouts are consumed by the GPU library (libbling_gpu.so) and, in
tests, by the CPU oracle; the descriptor is the flat hand-off that replaces
bling's closure records (Primitive.hs:21-27, Reflection.hs:42).
"""
from __future__ import annotations

import ctypes as C

BANDS = 16
F16 = C.c_float * BANDS
M16 = C.c_float * 16

BLING_OK = 0
BLING_ERR_INVALID_ARG = -1
BLING_ERR_OOM = -2
BLING_ERR_CUDA = -3
BLING_ERR_TIMEOUT = -4
BLING_ERR_BOUNDS = -5
BLING_ERR_STATE = -6

FLAG_WIDE_BVH = 1
FLAG_GPU_BVH = 2
FLAG_COMPACT_BVH = 4
FLAG_BIN_RAYS = 8

MAT_MATTE, MAT_PLASTIC, MAT_METAL, MAT_GLASS, MAT_MIRROR = 0, 1, 2, 3, 4
MAT_SHINY_METAL, MAT_TRANS_MATTE = 5, 6
MAT_SUBSTRATE, MAT_BLACKBODY = 7, 8  # substrate: ka in kt, urough in roughness, vrough in sigma, depth in ior
SHAPE_SPHERE, SHAPE_QUAD, SHAPE_BOX, SHAPE_DISK, SHAPE_CYLINDER = 0, 1, 2, 3, 4
LIGHT_DIRECTIONAL, LIGHT_POINT, LIGHT_INFINITE, LIGHT_SUNSKY = 0, 1, 2, 3
FILTER_BOX, FILTER_GAUSS, FILTER_MITCHELL, FILTER_SINC, FILTER_TRIANGLE = 0, 1, 2, 3, 4
SAMPLER_STRATIFIED, SAMPLER_RANDOM = 0, 1
ABI_VERSION = 5  # BLING_ABI_VERSION of include/bling_gpu.h


class Opts(C.Structure):
    _fields_ = [("device", C.c_int32), ("flags", C.c_uint32), ("block_size", C.c_int32),
                ("bvh_leaf_size", C.c_int32)]


class Material(C.Structure):
    _fields_ = [("kind", C.c_int32), ("sigma", C.c_float), ("roughness", C.c_float),
                ("ior", C.c_float), ("kd", F16), ("ks", F16), ("kt", F16), ("eta", F16),
                ("k", F16), ("kd_texture", C.c_int32), ("kd_tex_params", C.c_float * 9),
                ("kd2", F16), ("tex", C.c_int32 * 8), ("bump", C.c_int32),
                ("reserved_tex", C.c_int32)]


TEX_CONSTANT, TEX_CHECKER, TEX_GRAPH_PAPER = 0, 1, 2
# bling_material.tex slots
SLOT_KD, SLOT_KS, SLOT_KT, SLOT_ETA, SLOT_K, SLOT_SIGMA, SLOT_ROUGHNESS, SLOT_IOR = range(8)
# bling_texture kinds: spectrum-valued, then scalar-valued
TEXN_CONSTANT, TEXN_BLEND, TEXN_CHECKER, TEXN_GRAPH_PAPER, TEXN_GRADIENT, TEXN_IMAGE = range(6)
TEXN_SCALAR, TEXN_SCALE, TEXN_PERLIN, TEXN_FBM, TEXN_CELL_NOISE, TEXN_CRYSTAL, \
    TEXN_IMAGE_SCALAR = range(16, 23)
MAP_UV, MAP_PLANAR, MAP_IDENTITY3D = 0, 1, 2
DIST_EUCLIDIAN, DIST_EUCLIDIAN2, DIST_MANHATTAN, DIST_CHEBYSHEV = 0, 1, 2, 3
TEX_MAX_DEPTH = 8


class Texture(C.Structure):
    _fields_ = [("kind", C.c_int32), ("a", C.c_int32), ("b", C.c_int32), ("c", C.c_int32),
                ("ivalue", C.c_int32), ("map_kind", C.c_int32), ("map", C.c_float * 16),
                ("p", C.c_float * 4), ("spectrum", F16), ("data", C.POINTER(C.c_float)),
                ("pixels", C.POINTER(C.c_uint8)), ("width", C.c_int32), ("height", C.c_int32)]


class MeshDesc(C.Structure):
    _fields_ = [("vertices", C.POINTER(C.c_float)), ("n_vertices", C.c_int64),
                ("indices", C.POINTER(C.c_int32)), ("n_indices", C.c_int64),
                ("normals", C.POINTER(C.c_float)), ("uvs", C.POINTER(C.c_float)),
                ("material", C.c_int32), ("reserved", C.c_int32)]


class ShapeDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("material", C.c_int32), ("params", C.c_float * 6),
                ("o2w", M16), ("w2o", M16), ("emissive", C.c_int32), ("emission", F16)]


class LightDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("spectrum", F16), ("vec", C.c_float * 3),
                ("env", C.POINTER(C.c_float)), ("env_w", C.c_int32), ("env_h", C.c_int32),
                ("w2l", M16), ("l2w", M16), ("east", C.c_float * 3), ("turbidity", C.c_float)]


class CameraDesc(C.Structure):
    _fields_ = [("c2w", M16), ("c2w_inv", M16), ("r2c", M16), ("r2c_inv", M16),
                ("lens_radius", C.c_float), ("focal_distance", C.c_float),
                ("w2r", M16), ("pixel_area", C.c_float), ("reserved", C.c_float)]


class SceneDesc(C.Structure):
    _fields_ = [("meshes", C.POINTER(MeshDesc)), ("n_meshes", C.c_int32),
                ("shapes", C.POINTER(ShapeDesc)), ("n_shapes", C.c_int32),
                ("materials", C.POINTER(Material)), ("n_materials", C.c_int32),
                ("lights", C.POINTER(LightDesc)), ("n_lights", C.c_int32),
                ("prim_order", C.POINTER(C.c_int32)), ("camera", CameraDesc),
                ("textures", C.POINTER(Texture)), ("n_textures", C.c_int32),
                ("reserved_desc", C.c_int32)]


class RenderParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("strata_x", C.c_int32),
                ("strata_y", C.c_int32), ("max_depth", C.c_int32), ("sample_depth", C.c_int32),
                ("rr_depth", C.c_int32), ("filter_kind", C.c_int32),
                ("filter_params", C.c_float * 4), ("seed", C.c_uint64),
                ("sampler_kind", C.c_int32), ("reserved", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("rays_closest", C.c_uint64), ("rays_any", C.c_uint64),
                ("path_samples", C.c_uint64), ("nonfinite_drops", C.c_uint64),
                ("degenerate_rays", C.c_uint64),
                ("bvh_build_ms", C.c_double), ("last_pass_ms", C.c_double),
                ("bvh_nodes", C.c_uint64), ("bvh_leaf_prims", C.c_uint64),
                ("device_bytes", C.c_uint64), ("light_splats", C.c_uint64),
                ("scene_build_ms", C.c_double), ("nonfinite_pass", C.c_int64),
                ("nonfinite_pixel", C.c_int32 * 2), ("nonfinite_sample", C.c_int32),
                ("reserved_stats", C.c_int32)]


class SppmParams(C.Structure):
    """bling_sppm_params: mkSPPM n md r alpha, the pixel filter, the seed."""
    _fields_ = [("photons", C.c_int64), ("max_depth", C.c_int32), ("radius", C.c_float),
                ("alpha", C.c_float), ("filter_kind", C.c_int32), ("filter_params", C.c_float * 4),
                ("seed", C.c_uint64)]


def sppm_params(photons, max_depth=5, radius=0.05, alpha=0.7, filter_kind=FILTER_BOX,
                filter_params=(0.0, 0.0, 0.0, 0.0), seed=1) -> SppmParams:
    p = SppmParams()
    p.photons, p.max_depth, p.radius, p.alpha = photons, max_depth, radius, alpha
    p.filter_kind, p.seed = filter_kind, seed
    p.filter_params[:] = list(filter_params)
    return p


class LightParams(C.Structure):
    """bling_light_params: photons per pass, seed, depth limit (0: none)."""
    _fields_ = [("photons", C.c_int64), ("seed", C.c_uint64), ("max_depth", C.c_int32),
                ("reserved", C.c_int32)]


BATCH_PLAIN_LAUNCHES, BATCH_GRAPH, BATCH_DEVICE_LOOP = 0, 1, 2


class BatchOpts(C.Structure):
    _fields_ = [("slots", C.c_int64), ("block_size", C.c_int32), ("max_jobs", C.c_int32),
                ("sort_rays", C.c_int32), ("graph_mode", C.c_int32),
                ("iters_per_launch", C.c_int32), ("max_run_iterations", C.c_int32)]


class BatchStats(C.Structure):
    _fields_ = [("rays_closest", C.c_uint64), ("rays_any", C.c_uint64),
                ("path_samples", C.c_uint64), ("nonfinite_drops", C.c_uint64),
                ("degenerate_rays", C.c_uint64), ("iterations", C.c_uint64),
                ("samples_submitted", C.c_uint64), ("samples_started", C.c_uint64),
                ("jobs_submitted", C.c_int64), ("jobs_done", C.c_int64),
                ("jobs_active", C.c_int64), ("device_bytes", C.c_uint64)]


def fptr(a):
    """float* of a C-contiguous float32 numpy array (or NULL for None)."""
    if a is None:
        return C.POINTER(C.c_float)()
    assert a.dtype.name == "float32" and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_float))


def iptr(a):
    if a is None:
        return C.POINTER(C.c_int32)()
    assert a.dtype.name == "int32" and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class ServerOpts(C.Structure):
    _fields_ = [("batch", BatchOpts), ("hbm_budget_bytes", C.c_uint64),
                ("iters_per_step", C.c_int32), ("reserved", C.c_int32)]


class JobTimes(C.Structure):
    _fields_ = [("submitted", C.c_double), ("admitted", C.c_double), ("finished", C.c_double),
                ("samples", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [("jobs_submitted", C.c_int64), ("jobs_admitted", C.c_int64),
                ("jobs_done", C.c_int64), ("jobs_failed", C.c_int64),
                ("jobs_running", C.c_int64), ("jobs_pending", C.c_int64),
                ("samples_done", C.c_uint64), ("rays_closest", C.c_uint64),
                ("rays_any", C.c_uint64), ("iterations", C.c_uint64),
                ("budget_bytes", C.c_uint64), ("bytes_in_use", C.c_uint64),
                ("peak_bytes_in_use", C.c_uint64)]
FILM_FP64 = 1
