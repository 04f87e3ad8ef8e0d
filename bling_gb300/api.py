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

import ctypes as C
import weakref
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import abi

_LIB_PATH = Path(__file__).resolve().parent / "libbling_gpu.so"
_lib = None


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
    L.bling_film_destroy.argtypes = [vp]
    L.bling_film_clear.argtypes = [vp]
    L.bling_film_read.argtypes = [vp, P(C.c_float)]
    L.bling_film_resolve.argtypes = [vp, P(C.c_float)]
    L.bling_render_pass.argtypes = [vp, vp, P(abi.RenderParams), C.c_uint64]
    L.bling_rgb_to_spectrum.argtypes = [C.c_int32, C.c_float, C.c_float, C.c_float, P(C.c_float)]
    L.bling_spectrum_to_xyz.argtypes = [P(C.c_float), P(C.c_float)]
    for fn in ("bling_ctx_create", "bling_ctx_set_stream", "bling_scene_create", "bling_scene_stats",
               "bling_trace_closest", "bling_trace_any", "bling_trace_closest_device",
               "bling_trace_any_device", "bling_film_create", "bling_film_clear", "bling_film_read",
               "bling_film_resolve", "bling_render_pass"):
        getattr(L, fn).restype = C.c_int
    _lib = L
    return L


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Context:
    """A CUDA device plus one stream (``bling_ctx``)."""

    def __init__(self, device: int = 0, block_size: int = 0, bvh_leaf_size: int = 0,
                 wide_bvh: bool = False):
        L = lib()
        o = abi.Opts()
        o.device, o.block_size, o.bvh_leaf_size = device, block_size, bvh_leaf_size
        o.flags = abi.FLAG_WIDE_BVH if wide_bvh else 0
        self.h = C.c_void_p()
        self._children = weakref.WeakSet()  # scenes and films, closed before the context
        rc = L.bling_ctx_create(C.byref(self.h), C.byref(o))
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

    def film(self, width: int, height: int) -> "Film":
        return Film(self, width, height)


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
        return {k: getattr(s, k) for k, _ in abi.Stats._fields_}

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

    def render_pass(self, film: "Film", params, pass_index: int = 0):
        self.ctx.check(lib().bling_render_pass(self.h, film.h, C.byref(params), pass_index))


class Film:
    """A (weight, X, Y, Z) film resident on the device (Image.hs:64-82)."""

    def __init__(self, ctx: Context, width: int, height: int):
        self.ctx, self.width, self.height = ctx, width, height
        self.h = C.c_void_p()
        ctx.check(lib().bling_film_create(ctx.h, width, height, C.byref(self.h)))
        ctx._children.add(self)

    def close(self):
        if getattr(self, "h", None):
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
