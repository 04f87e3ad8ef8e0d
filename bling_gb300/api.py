"""Python binding of the GB300 path-tracing core (ctypes over libbling_gpu.so).

Mirrors the reference's drop-in point: :class:`GpuPathRenderer` implements the
``Renderer`` contract of bling (``render :: a -> RenderJob -> ProgressReporter
-> IO ()``, Rendering.hs:77-78) the way ``prender`` does (Rendering.hs:111-140):
one pass after another, each adding ``strata_x * strata_y`` samples per pixel
to the film, a ``PassDone`` progress event after every pass, and stopping
when the reporter returns False.

The extension is required: importing works without it, but every call that
needs it raises :class:`BlingUnavailable`; nothing falls back to the CPU.
"""
from __future__ import annotations

import atexit
import ctypes as C
import weakref
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import abi

_LIB_PATH = Path(__file__).resolve().parent / "libbling_gpu.so"
_lib = None
_live_contexts = weakref.WeakSet()


@atexit.register
def _close_all():
    """Closes every live context (its scenes, films, batches and servers
    first) while the interpreter and the CUDA runtime are still intact: at
    interpreter teardown, objects are finalized in no fixed order."""
    for ctx in list(_live_contexts):
        try:
            ctx.close()
        except Exception:  # noqa: BLE001 - best effort at exit
            pass


class BlingError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"bling error {code}: {msg}")
        self.code = code


class BlingUnavailable(BlingError):
    pass


def lib():
    """Loads the in-tree CUDA library (built by bling_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        raise BlingUnavailable(-3, f"{_LIB_PATH.name} is not built; run bling_gb300.build.build()")
    L = C.CDLL(str(_LIB_PATH))
    P, vp = C.POINTER, C.c_void_p
    L.bling_abi_version.restype = C.c_int
    if L.bling_abi_version() != abi.ABI_VERSION:
        raise BlingUnavailable(-3, f"{_LIB_PATH.name} has ABI version {L.bling_abi_version()}, "
                               f"the bindings expect {abi.ABI_VERSION}: rebuild it")
    L.bling_ctx_create.argtypes = [P(vp), P(abi.Opts)]
    L.bling_ctx_destroy.argtypes = [vp]
    L.bling_last_error.argtypes = [vp]
    L.bling_last_error.restype = C.c_char_p
    L.bling_ctx_set_stream.argtypes = [vp, vp]
    L.bling_scene_create.argtypes = [vp, P(abi.SceneDesc), P(vp)]
    L.bling_scene_destroy.argtypes = [vp]
    L.bling_scene_stats.argtypes = [vp, P(abi.Stats)]
    L.bling_trace_closest.argtypes = [vp, P(C.c_float), C.c_size_t, P(C.c_float), P(C.c_int32),
                                      P(C.c_float)]
    L.bling_trace_any.argtypes = [vp, P(C.c_float), C.c_size_t, P(C.c_uint8)]
    L.bling_trace_closest_device.argtypes = [vp, vp, C.c_size_t, vp, vp, vp]
    L.bling_trace_any_device.argtypes = [vp, vp, C.c_size_t, vp]
    L.bling_trace_counts.argtypes = [vp, P(C.c_float), C.c_size_t, P(C.c_uint64), P(C.c_uint64)]
    L.bling_trace_counts.restype = C.c_int
    L.bling_film_create.argtypes = [vp, C.c_int32, C.c_int32, P(vp)]
    L.bling_film_create_ex.argtypes = [vp, C.c_int32, C.c_int32, C.c_uint32, P(vp)]
    L.bling_film_fold.argtypes = [vp]
    L.bling_film_read_f64.argtypes = [vp, P(C.c_double)]
    for fn in ("bling_film_create_ex", "bling_film_fold", "bling_film_read_f64"):
        getattr(L, fn).restype = C.c_int
    L.bling_film_destroy.argtypes = [vp]
    L.bling_film_clear.argtypes = [vp]
    L.bling_film_read.argtypes = [vp, P(C.c_float)]
    L.bling_film_resolve.argtypes = [vp, P(C.c_float)]
    L.bling_render_pass.argtypes = [vp, vp, P(abi.RenderParams), C.c_uint64]
    L.bling_render_pass_camera.argtypes = [vp, vp, P(abi.RenderParams), P(abi.CameraDesc),
                                           C.c_uint64]
    L.bling_render_pass_camera.restype = C.c_int
    L.bling_light_pass.argtypes = [vp, vp, P(abi.LightParams), C.c_uint64]
    L.bling_film_read_splats.argtypes = [vp, P(C.c_float)]
    L.bling_film_resolve_splats.argtypes = [vp, C.c_float, P(C.c_float)]
    L.bling_sppm_pass.argtypes = [vp, vp, P(abi.SppmParams), C.c_uint64]
    L.bling_film_read_sppm_radii.argtypes = [vp, P(C.c_float), C.c_int64, P(C.c_int64)]
    for fn in ("bling_light_pass", "bling_film_read_splats", "bling_film_resolve_splats",
               "bling_sppm_pass", "bling_film_read_sppm_radii"):
        getattr(L, fn).restype = C.c_int
    L.bling_rgb_to_spectrum.argtypes = [C.c_int32, C.c_float, C.c_float, C.c_float, P(C.c_float)]
    L.bling_spectrum_to_xyz.argtypes = [P(C.c_float), P(C.c_float)]
    L.bling_sunsky_eval.argtypes = [P(C.c_float), P(C.c_float), C.c_float, C.c_float, C.c_float,
                                    P(C.c_float)]
    L.bling_batch_create.argtypes = [vp, P(abi.BatchOpts), P(vp)]
    L.bling_batch_destroy.argtypes = [vp]
    L.bling_batch_submit.argtypes = [vp, vp, vp, P(abi.RenderParams), P(abi.CameraDesc), C.c_uint64,
                                     P(C.c_int64)]
    L.bling_batch_step.argtypes = [vp, C.c_int32]
    L.bling_batch_run.argtypes = [vp]
    L.bling_batch_job_status.argtypes = [vp, C.c_int64, P(C.c_uint64), P(C.c_uint64)]
    L.bling_batch_stats_get.argtypes = [vp, P(abi.BatchStats)]
    L.bling_server_create.argtypes = [vp, P(abi.ServerOpts), P(vp)]
    L.bling_server_destroy.argtypes = [vp]
    L.bling_server_submit.argtypes = [vp, vp, P(abi.RenderParams), P(abi.CameraDesc), C.c_uint64,
                                      P(C.c_int64)]
    L.bling_server_wait.argtypes = [vp, C.c_int64, C.c_int32, P(C.c_float), P(abi.JobTimes)]
    L.bling_server_stats_get.argtypes = [vp, P(abi.ServerStats)]
    L.bling_server_last_error.argtypes = [vp]
    L.bling_server_last_error.restype = C.c_char_p
    L.bling_server_debug_fail_step.argtypes = [vp, C.c_int32]
    for fn in ("bling_server_create", "bling_server_submit", "bling_server_wait",
               "bling_server_stats_get", "bling_server_debug_fail_step"):
        getattr(L, fn).restype = C.c_int
    for fn in ("bling_ctx_create", "bling_ctx_set_stream", "bling_scene_create", "bling_scene_stats",
               "bling_trace_closest", "bling_trace_any", "bling_trace_closest_device",
               "bling_trace_any_device", "bling_film_create", "bling_film_clear", "bling_film_read",
               "bling_film_resolve", "bling_render_pass", "bling_batch_create", "bling_batch_submit",
               "bling_batch_step", "bling_batch_run", "bling_batch_job_status",
               "bling_batch_stats_get"):
        getattr(L, fn).restype = C.c_int
    _lib = L
    return L


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Context:
    """A CUDA device plus one stream (``bling_ctx``)."""

    def __init__(self, device: int = 0, block_size: int = 0, bvh_leaf_size: int = 0,
                 wide_bvh: bool = False, gpu_bvh: bool = False, compact_bvh: bool = False,
                 bin_rays: bool = False):
        """gpu_bvh: scenes build their BVH on the GPU (BLING_FLAG_GPU_BVH);
        compact_bvh: 32-byte quantised binary nodes (BLING_FLAG_COMPACT_BVH);
        bin_rays: Morton-ordered bounce rays in render passes (BLING_FLAG_BIN_RAYS)"""
        L = lib()
        o = abi.Opts()
        o.device, o.block_size, o.bvh_leaf_size = device, block_size, bvh_leaf_size
        o.flags = ((abi.FLAG_WIDE_BVH if wide_bvh else 0) | (abi.FLAG_GPU_BVH if gpu_bvh else 0) |
                   (abi.FLAG_COMPACT_BVH if compact_bvh else 0) |
                   (abi.FLAG_BIN_RAYS if bin_rays else 0))
        self.wide_bvh = wide_bvh
        self.gpu_bvh = gpu_bvh
        self.compact_bvh = compact_bvh
        self.h = C.c_void_p()
        self._children = weakref.WeakSet()  # scenes and films, closed before the context
        rc = L.bling_ctx_create(C.byref(self.h), C.byref(o))
        _live_contexts.add(self)
        if rc != 0:
            msg = L.bling_last_error(self.h).decode() if self.h else "context creation failed"
            if self.h:
                L.bling_ctx_destroy(self.h)
                self.h = None
            raise BlingUnavailable(rc, msg)

    def check(self, rc: int):
        if rc != 0:
            raise BlingError(rc, lib().bling_last_error(self.h).decode())

    def set_stream(self, stream_handle: int | None):
        """Enqueue work on an external cudaStream_t (e.g. torch.cuda.current_stream().cuda_stream)."""
        self.check(lib().bling_ctx_set_stream(self.h, C.c_void_p(stream_handle or 0)))

    def close(self):
        if getattr(self, "h", None):
            for child in list(self._children):
                child.close()
            lib().bling_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass

    def scene(self, scene) -> "GpuScene":
        return GpuScene(self, scene)

    def film(self, width: int, height: int, fp64: bool = False) -> "Film":
        return Film(self, width, height, fp64)


class GpuScene:
    """A scene resident on the device: BVH, primitives, materials, lights."""

    def __init__(self, ctx: Context, scene):
        self.ctx = ctx
        desc, keep = scene.desc()
        self.h = C.c_void_p()
        ctx.check(lib().bling_scene_create(ctx.h, C.byref(desc), C.byref(self.h)))
        ctx._children.add(self)

    def close(self):
        if getattr(self, "h", None):
            if getattr(self.ctx, "h", None):  # a destroyed context took its objects' handles with it
                lib().bling_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def stats(self) -> dict:
        s = abi.Stats()
        self.ctx.check(lib().bling_scene_stats(self.h, C.byref(s)))
        out = {k: getattr(s, k) for k, _ in abi.Stats._fields_ if k != "reserved_stats"}
        out["nonfinite_pixel"] = tuple(s.nonfinite_pixel)
        return out

    # --- ray queries over host arrays (SoA float32 (8, n)) ---
    def closest(self, rays: np.ndarray, with_bary: bool = True):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        assert rays.ndim == 2 and rays.shape[0] == 8
        n = rays.shape[1]
        t = np.empty(n, np.float32)
        prim = np.empty(n, np.int32)
        b = np.empty(2 * n, np.float32) if with_bary else None
        self.ctx.check(lib().bling_trace_closest(
            self.h, _fp(rays), n, _fp(t), prim.ctypes.data_as(C.POINTER(C.c_int32)),
            _fp(b) if b is not None else C.POINTER(C.c_float)()))
        return t, prim, (b.reshape(n, 2) if b is not None else None)

    def any(self, rays: np.ndarray):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[1]
        hit = np.empty(n, np.uint8)
        self.ctx.check(lib().bling_trace_any(self.h, _fp(rays), n,
                                             hit.ctypes.data_as(C.POINTER(C.c_uint8))))
        return hit

    def traversal_counts(self, rays: np.ndarray) -> dict:
        """Mean BVH nodes visited and leaf primitives tested per closest-hit ray."""
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[1]
        nodes, prims = C.c_uint64(), C.c_uint64()
        self.ctx.check(lib().bling_trace_counts(self.h, _fp(rays), n, C.byref(nodes), C.byref(prims)))
        return {"nodes_per_ray": nodes.value / max(1, n), "slots_per_ray": prims.value / max(1, n)}

    # --- ray queries over device buffers (torch CUDA tensors) ---
    def closest_device(self, d_rays, d_t, d_prim, d_b=None):
        n = d_rays.shape[-1]
        self.ctx.check(lib().bling_trace_closest_device(
            self.h, C.c_void_p(d_rays.data_ptr()), n, C.c_void_p(d_t.data_ptr()),
            C.c_void_p(d_prim.data_ptr()), C.c_void_p(d_b.data_ptr() if d_b is not None else 0)))

    def any_device(self, d_rays, d_hit):
        n = d_rays.shape[-1]
        self.ctx.check(lib().bling_trace_any_device(self.h, C.c_void_p(d_rays.data_ptr()), n,
                                                    C.c_void_p(d_hit.data_ptr())))

    def render_pass(self, film: "Film", params, pass_index: int = 0, camera=None):
        """one pass into the film; camera: an abi.CameraDesc (None: the scene's)"""
        if camera is None:
            self.ctx.check(lib().bling_render_pass(self.h, film.h, C.byref(params), pass_index))
        else:
            self.ctx.check(lib().bling_render_pass_camera(self.h, film.h, C.byref(params),
                                                          C.byref(camera), pass_index))

    def light_pass(self, film: "Film", photons: int, seed: int = 0, pass_index: int = 0,
                   max_depth: int = 0):
        """one light-tracer pass of `photons` photons into the film's splat
        image (LightTracer.hs:37-110); max_depth 0: no limit"""
        p = abi.LightParams()
        p.photons, p.seed, p.max_depth = photons, seed, max_depth
        self.ctx.check(lib().bling_light_pass(self.h, film.h, C.byref(p), pass_index))

    def sppm_pass(self, film: "Film", params, pass_index: int = 0):
        """one SPPM pass (SPPM.hs:410-480): camera samples into the film,
        photon splats into its splat image; params: abi.SppmParams"""
        self.ctx.check(lib().bling_sppm_pass(self.h, film.h, C.byref(params), pass_index))


class Film:
    """A (weight, X, Y, Z) film resident on the device (Image.hs:64-82)."""

    def __init__(self, ctx: Context, width: int, height: int, fp64: bool = False):
        self.ctx, self.width, self.height, self.fp64 = ctx, width, height, fp64
        self.h = C.c_void_p()
        ctx.check(lib().bling_film_create_ex(ctx.h, width, height,
                                             abi.FILM_FP64 if fp64 else 0, C.byref(self.h)))
        ctx._children.add(self)

    def fold(self):
        """adds the FP32 samples into the FP64 totals (BLING_FILM_FP64 films)"""
        self.ctx.check(lib().bling_film_fold(self.h))

    def read_f64(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 4), np.float64)
        self.ctx.check(lib().bling_film_read_f64(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def close(self):
        if getattr(self, "h", None):
            if getattr(self.ctx, "h", None):  # a destroyed context took its objects' handles with it
                lib().bling_film_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def clear(self):
        self.ctx.check(lib().bling_film_clear(self.h))

    def read(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 4), np.float32)
        self.ctx.check(lib().bling_film_read(self.h, _fp(out)))
        return out

    def resolve(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 3), np.float32)
        self.ctx.check(lib().bling_film_resolve(self.h, _fp(out)))
        return out

    def read_splats(self) -> np.ndarray:
        """the (height, width, 3) XYZ splat image of light passes"""
        out = np.empty((self.height, self.width, 3), np.float32)
        self.ctx.check(lib().bling_film_read_splats(self.h, _fp(out)))
        return out

    def read_sppm_radii(self) -> np.ndarray:
        """the squared SPPM radii of the sample extent's pixels (empty before
        the first SPPM pass)"""
        n = C.c_int64()
        self.ctx.check(lib().bling_film_read_sppm_radii(self.h, None, 0, C.byref(n)))
        out = np.empty(n.value, np.float32)
        if n.value:
            self.ctx.check(lib().bling_film_read_sppm_radii(self.h, _fp(out), n.value, C.byref(n)))
        return out

    def resolve_splats(self, splat_weight: float) -> np.ndarray:
        """getPixel with splat weight (Image.hs:302-315) to linear sRGB"""
        out = np.empty((self.height, self.width, 3), np.float32)
        self.ctx.check(lib().bling_film_resolve_splats(self.h, splat_weight, _fp(out)))
        return out


class Batch:
    """Many render jobs in one persistent wavefront (``bling_batch``).

    A job is one pass (``GpuScene.render_pass``) of a scene into a film; jobs
    may be submitted between steps while others are in flight."""

    def __init__(self, ctx: Context, slots: int = 0, block_size: int = 0, max_jobs: int = 0,
                 sort_rays: bool = False, graph_mode: int = abi.BATCH_GRAPH,
                 iters_per_launch: int = 0, max_run_iterations: int = 0):
        self.ctx = ctx
        o = abi.BatchOpts()
        o.slots, o.block_size, o.max_jobs = slots, block_size, max_jobs
        o.sort_rays, o.graph_mode, o.iters_per_launch = int(sort_rays), graph_mode, iters_per_launch
        o.max_run_iterations = max_run_iterations
        self.h = C.c_void_p()
        ctx.check(lib().bling_batch_create(ctx.h, C.byref(o), C.byref(self.h)))
        ctx._children.add(self)

    def close(self):
        if getattr(self, "h", None):
            if getattr(self.ctx, "h", None):  # a destroyed context took its objects' handles with it
                lib().bling_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def submit(self, scene: GpuScene, film: Film, params, pass_index: int = 0,
               camera=None) -> int:
        """camera: an abi.CameraDesc for this job (None: the scene's camera)."""
        job = C.c_int64()
        cam = C.byref(camera) if camera is not None else None
        self.ctx.check(lib().bling_batch_submit(self.h, scene.h, film.h, C.byref(params), cam,
                                                pass_index, C.byref(job)))
        return job.value

    def step(self, iterations: int = 1):
        self.ctx.check(lib().bling_batch_step(self.h, iterations))

    def run(self):
        self.ctx.check(lib().bling_batch_run(self.h))

    def status(self, job: int) -> tuple[int, int]:
        done, total = C.c_uint64(), C.c_uint64()
        self.ctx.check(lib().bling_batch_job_status(self.h, job, C.byref(done), C.byref(total)))
        return done.value, total.value

    def done(self, job: int) -> bool:
        d, t = self.status(job)
        return d == t

    def stats(self) -> dict:
        s = abi.BatchStats()
        self.ctx.check(lib().bling_batch_stats_get(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in abi.BatchStats._fields_}


class Server:
    """Continuous batching of render jobs (``bling_server``): submit from any
    thread, wait for the film.  The context must outlive the server."""

    def __init__(self, ctx: Context, hbm_budget_bytes: int = 0, iters_per_step: int = 0,
                 slots: int = 0, block_size: int = 0, max_jobs: int = 0, sort_rays: bool = False,
                 graph_mode: int = 0, iters_per_launch: int = 0):
        self.ctx = ctx
        o = abi.ServerOpts()
        o.batch.slots, o.batch.block_size, o.batch.max_jobs = slots, block_size, max_jobs
        o.batch.sort_rays, o.batch.graph_mode = int(sort_rays), graph_mode
        o.batch.iters_per_launch = iters_per_launch
        o.hbm_budget_bytes, o.iters_per_step = hbm_budget_bytes, iters_per_step
        self.h = C.c_void_p()
        ctx.check(lib().bling_server_create(ctx.h, C.byref(o), C.byref(self.h)))
        ctx._children.add(self)
        self._sizes = {}

    def _check(self, rc):
        if rc != 0:
            raise BlingError(rc, lib().bling_server_last_error(self.h).decode())

    def debug_fail_step(self, after_steps: int):
        """Test hook: the wavefront step after `after_steps` more steps fails
        on the host (``bling_server_debug_fail_step``); -1 disarms."""
        self._check(lib().bling_server_debug_fail_step(self.h, after_steps))

    def close(self):
        if getattr(self, "h", None):
            if getattr(self.ctx, "h", None):  # a destroyed context took its objects' handles with it
                lib().bling_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def submit(self, scene: GpuScene, params, pass_index: int = 0, camera=None) -> int:
        t = C.c_int64()
        cam = C.byref(camera) if camera is not None else None
        self._check(lib().bling_server_submit(self.h, scene.h, C.byref(params), cam, pass_index,
                                              C.byref(t)))
        self._sizes[t.value] = (params.height, params.width)
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1, want_film: bool = True):
        """(film (h, w, 4) float32 or None, times dict)"""
        size = self._sizes.get(ticket)  # None: not submitted here; the library reports it
        film = np.empty((*size, 4), np.float32) if want_film and size else None
        times = abi.JobTimes()
        rc = lib().bling_server_wait(self.h, ticket, timeout_ms,
                                     _fp(film) if film is not None else None, C.byref(times))
        if rc != abi.BLING_ERR_TIMEOUT:
            self._sizes.pop(ticket, None)
        self._check(rc)
        return film, {k: getattr(times, k) for k, _ in abi.JobTimes._fields_}

    def stats(self) -> dict:
        s = abi.ServerStats()
        self._check(lib().bling_server_stats_get(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in abi.ServerStats._fields_}


# ---------------------------------------------------------------- Renderer
@dataclass
class RenderJob:
    """RenderJob (Rendering.hs:37-44): scene, pixel filter and image size,
    here with the sampler/integrator settings of the job."""
    scene: object
    params: object  # abi.RenderParams


@dataclass
class PassDone:
    """Progress event after each pass (Rendering.hs:69-73)."""
    pass_num: int
    film: Film
    splat_weight: float = 1.0


class GpuLightTracer:
    """``mkLightTracer ppp`` as a bling ``Renderer`` (LightTracer.hs:37-44):
    pass n adds ppp photons to the film's splat image and reports the splat
    weight 1 / (n ppp).  max_depth 0 keeps the reference's unbounded paths."""

    def __init__(self, photons_per_pass: int, ctx: Context | None = None, seed: int = 0,
                 max_depth: int = 0):
        self.ctx = ctx or Context()
        self.ppp, self.seed, self.max_depth = photons_per_pass, seed, max_depth

    def render(self, job: RenderJob, report) -> Film:
        p = job.params
        gscene = job.scene if isinstance(job.scene, GpuScene) else self.ctx.scene(job.scene)
        film = self.ctx.film(p.width, p.height)
        report("Started")
        n = 1
        while True:
            gscene.light_pass(film, self.ppp, seed=self.seed, pass_index=n, max_depth=self.max_depth)
            if not report(PassDone(n, film, 1.0 / (n * self.ppp))):
                break
            n += 1
        return film


class GpuSPPM:
    """``mkSPPM n md r alpha`` as a bling ``Renderer`` (SPPM.hs:466-480): pass
    n adds camera samples to the film and ceil(sqrt n)^2 photons' splats to
    its splat image, shrinks the radii, and reports the splat weight
    1 / (n sn^2).  The job's pixel filter applies to the camera samples."""

    def __init__(self, photons: int, max_depth: int, radius: float, alpha: float = 0.8,
                 ctx: Context | None = None, seed: int = 1):
        self.ctx = ctx or Context()
        self.photons, self.max_depth, self.radius, self.alpha, self.seed = (photons, max_depth,
                                                                            radius, alpha, seed)

    def render(self, job: RenderJob, report) -> Film:
        p = job.params
        gscene = job.scene if isinstance(job.scene, GpuScene) else self.ctx.scene(job.scene)
        film = self.ctx.film(p.width, p.height)
        sp = abi.sppm_params(self.photons, self.max_depth, self.radius, self.alpha,
                             filter_kind=p.filter_kind, filter_params=tuple(p.filter_params),
                             seed=self.seed)
        sn = max(1, int(np.ceil(np.sqrt(np.float32(self.photons)))))
        report("Started")
        n = 1
        while True:
            gscene.sppm_pass(film, sp, n - 1)
            if not report(PassDone(n, film, 1.0 / (n * sn * sn))):
                break
            n += 1
        return film


class GpuPathRenderer:
    """The GPU path integrator as a bling ``Renderer`` (Rendering.hs:77-78)."""

    def __init__(self, ctx: Context | None = None):
        self.ctx = ctx or Context()

    def render(self, job: RenderJob, report) -> Film:
        p = job.params
        gscene = job.scene if isinstance(job.scene, GpuScene) else self.ctx.scene(job.scene)
        film = self.ctx.film(p.width, p.height)
        report("Started")
        pass_num = 1
        while True:  # onePass (Rendering.hs:127-138)
            gscene.render_pass(film, p, pass_num)
            if not report(PassDone(pass_num, film, 1.0)):
                break
            pass_num += 1
        return film
