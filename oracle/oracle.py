"""ctypes wrapper of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
"""
from __future__ import annotations

import ctypes as C
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

from bling_gb300 import abi  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        from oracle.build import build  # noqa: WPS433
        path = build()
        L = C.CDLL(str(path))
        P = C.POINTER
        L.orc_scene_create.argtypes = [P(abi.SceneDesc), P(C.c_void_p)]
        L.orc_scene_destroy.argtypes = [C.c_void_p]
        L.orc_scene_prim_count.argtypes = [C.c_void_p]
        L.orc_scene_prim_count.restype = C.c_int64
        for fn in ("orc_trace_closest_brute", "orc_trace_closest_bvh"):
            getattr(L, fn).argtypes = [C.c_void_p, P(C.c_float), C.c_size_t, P(C.c_float),
                                       P(C.c_int32), P(C.c_float), C.c_int]
        for fn in ("orc_trace_any_brute", "orc_trace_any_bvh"):
            getattr(L, fn).argtypes = [C.c_void_p, P(C.c_float), C.c_size_t, P(C.c_uint8), C.c_int]
        L.orc_kdtree_build.argtypes = [C.c_void_p, C.c_int, P(C.c_int64)]
        L.orc_trace_closest_kd.argtypes = [C.c_void_p, P(C.c_float), C.c_size_t, P(C.c_float),
                                           P(C.c_int32), P(C.c_float), C.c_int, P(C.c_uint64)]
        L.orc_trace_any_kd.argtypes = [C.c_void_p, P(C.c_float), C.c_size_t, P(C.c_uint8),
                                       C.c_int, P(C.c_uint64)]
        L.orc_scene_use_kdtree.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.orc_render_pass.argtypes = [C.c_void_p, P(abi.RenderParams), C.c_uint64, P(C.c_float),
                                      C.c_int, C.c_int, C.c_int, P(C.c_uint64), P(C.c_uint64),
                                      P(C.c_uint64)]
        L.orc_render_pass_f64.argtypes = [C.c_void_p, P(abi.RenderParams), C.c_uint64,
                                          P(C.c_double), C.c_int, P(C.c_uint64)]
        L.orc_light_pass.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_uint64, C.c_uint64,
                                     C.c_int32, C.c_int64, C.c_int64, P(C.c_float), C.c_int,
                                     P(C.c_uint64)]
        L.orc_sppm_pass.argtypes = [C.c_void_p, P(abi.SppmParams), C.c_int32, C.c_int32,
                                    C.c_uint64, P(C.c_float), P(C.c_float), P(C.c_float),
                                    P(C.c_float), P(C.c_uint32), C.c_int64, C.c_int,
                                    P(C.c_uint64)]
        L.orc_sample_li.argtypes = [C.c_void_p, P(abi.RenderParams), C.c_uint64, C.c_int, C.c_int,
                                    C.c_int, P(C.c_float), P(C.c_float), P(C.c_float)]
        L.orc_rgb_to_spectrum.argtypes = [C.c_int, C.c_float, C.c_float, C.c_float, P(C.c_float)]
        L.orc_sunsky_eval.argtypes = [P(C.c_float), P(C.c_float), C.c_float, C.c_float, C.c_float,
                                      P(C.c_float)]
        L.orc_spectrum_to_xyz.argtypes = [P(C.c_float), P(C.c_float)]
        L.orc_texture_eval.argtypes = [C.c_void_p, C.c_int, P(C.c_float), C.c_float, C.c_float,
                                       P(C.c_float)]
        L.orc_xyz_to_rgb.argtypes = [P(C.c_float), P(C.c_float)]
        L.orc_filter_eval.argtypes = [C.c_int, P(C.c_float), C.c_float, C.c_float]
        L.orc_filter_eval.restype = C.c_float
        L.orc_filter_table.argtypes = [C.c_int, P(C.c_float), P(C.c_float)]
        L.orc_random_floats.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_int, C.c_uint32,
                                        C.c_uint32, C.c_int, P(C.c_float)]
        L.orc_permute.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
        L.orc_permute.restype = C.c_uint32
        L.orc_xf_translate.argtypes = [C.c_float, C.c_float, C.c_float, P(C.c_float)]
        L.orc_xf_scale.argtypes = [C.c_float, C.c_float, C.c_float, P(C.c_float)]
        L.orc_xf_rotate.argtypes = [C.c_int, C.c_float, P(C.c_float)]
        L.orc_xf_look_at.argtypes = [P(C.c_float), P(C.c_float), P(C.c_float), P(C.c_float)]
        L.orc_xf_perspective.argtypes = [C.c_float, C.c_float, C.c_float, P(C.c_float)]
        L.orc_xf_concat.argtypes = [P(C.c_float), P(C.c_float), P(C.c_float)]
        L.orc_camera_perspective.argtypes = [P(C.c_float), C.c_float, C.c_float, C.c_float,
                                             C.c_float, C.c_float, P(abi.CameraDesc)]
        _lib = L
    return _lib


def fp(a):
    return abi.fptr(a)


class OracleScene:
    def __init__(self, scene):
        self._desc, self._keep = scene.desc()
        self.kinds = [t.kind for t in getattr(scene, "textures", [])]
        self.h = C.c_void_p()
        rc = lib().orc_scene_create(C.byref(self._desc), C.byref(self.h))
        if rc != 0:
            raise ValueError(f"orc_scene_create failed: {rc}")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_scene_destroy(self.h)
            self.h = None

    @property
    def prim_count(self) -> int:
        return lib().orc_scene_prim_count(self.h)

    def closest(self, rays, brute=False, nthreads=0):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[1]
        t = np.empty(n, np.float32)
        prim = np.empty(n, np.int32)
        b = np.empty(2 * n, np.float32)
        fn = lib().orc_trace_closest_brute if brute else lib().orc_trace_closest_bvh
        fn(self.h, fp(rays), n, fp(t), prim.ctypes.data_as(C.POINTER(C.c_int32)), fp(b), nthreads)
        return t, prim, b.reshape(n, 2)

    def any(self, rays, brute=False, nthreads=0):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[1]
        hit = np.empty(n, np.uint8)
        fn = lib().orc_trace_any_brute if brute else lib().orc_trace_any_bvh
        fn(self.h, fp(rays), n, hit.ctypes.data_as(C.POINTER(C.c_uint8)), nthreads)
        return hit

    KD_STATS = ("interiors", "leaves", "empty_leaves", "leaf_refs", "max_leaf", "max_depth",
                "depth_sum", "depth_limit")

    def kdtree(self, nthreads=0) -> dict:
        """Builds the reference's kd-tree (once) and returns its statistics."""
        st = (C.c_int64 * 8)()
        lib().orc_kdtree_build(self.h, nthreads, st)
        return dict(zip(self.KD_STATS, list(st)))

    def closest_kd(self, rays, nthreads=0):
        """closest hits through the kd-tree in the reference's traversal
        order; returns (t, prim, b1b2, {"nodes": .., "prims": ..})"""
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[1]
        t = np.empty(n, np.float32)
        prim = np.empty(n, np.int32)
        b = np.empty(2 * n, np.float32)
        cnt = (C.c_uint64 * 2)()
        lib().orc_trace_closest_kd(self.h, fp(rays), n, fp(t),
                                   prim.ctypes.data_as(C.POINTER(C.c_int32)), fp(b), nthreads, cnt)
        return t, prim, b.reshape(n, 2), {"nodes": cnt[0], "prims": cnt[1]}

    def any_kd(self, rays, nthreads=0):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[1]
        hit = np.empty(n, np.uint8)
        cnt = (C.c_uint64 * 2)()
        lib().orc_trace_any_kd(self.h, fp(rays), n, hit.ctypes.data_as(C.POINTER(C.c_uint8)),
                               nthreads, cnt)
        return hit, {"nodes": cnt[0], "prims": cnt[1]}

    def use_kdtree(self, on=True, nthreads=0):
        """the renderers trace through the kd-tree (True) or the oracle's BVH"""
        lib().orc_scene_use_kdtree(self.h, int(bool(on)), nthreads)

    def render_pass(self, params, pass_index=0, film=None, rows=None, nthreads=0):
        if film is None:
            film = np.zeros((params.height, params.width, 4), np.float32)
        ps, rc_, ra = C.c_uint64(), C.c_uint64(), C.c_uint64()
        rb, re = rows if rows is not None else (0, 0)
        rc = lib().orc_render_pass(self.h, C.byref(params), pass_index, fp(film), rb, re, nthreads,
                                   C.byref(ps), C.byref(rc_), C.byref(ra))
        if rc != 0:
            raise ValueError(f"orc_render_pass failed: {rc}")
        return film, {"path_samples": ps.value, "rays_closest": rc_.value, "rays_any": ra.value}

    def render_pass_f64(self, params, pass_index=0, film=None, nthreads=0):
        """render_pass into a float64 film (tile and film sums in double)"""
        if film is None:
            film = np.zeros((params.height, params.width, 4), np.float64)
        assert film.dtype == np.float64 and film.flags.c_contiguous
        ps = C.c_uint64()
        rc = lib().orc_render_pass_f64(self.h, C.byref(params), pass_index,
                                       film.ctypes.data_as(C.POINTER(C.c_double)), nthreads,
                                       C.byref(ps))
        if rc != 0:
            raise ValueError(f"orc_render_pass_f64 failed: {rc}")
        return film, {"path_samples": ps.value}

    def light_pass(self, width, height, photons, seed=0, pass_index=0, max_depth=0, splats=None,
                   first=0, count=None, nthreads=0):
        """Photons [first, first + count) of a light-tracer pass into an
        (height, width, 3) XYZ splat image; returns (splats, stats)."""
        if splats is None:
            splats = np.zeros((height, width, 3), np.float32)
        count = photons - first if count is None else count
        st = (C.c_uint64 * 4)()
        rc = lib().orc_light_pass(self.h, width, height, seed, pass_index, max_depth, first, count,
                                  fp(splats), nthreads, st)
        if rc != 0:
            raise ValueError(f"orc_light_pass failed: {rc}")
        return splats, {"rays_closest": st[0], "rays_any": st[1], "splats": st[2],
                        "nonfinite": st[3]}

    def sppm_state(self, params, width, height):
        """fresh per-pixel SPPM statistics: radius^2 = r^2, N = 0, M = 0 over
        the sample extent (imageWindow')"""
        from bling_gb300.scene import render_params
        rp = render_params(width, height, (1, 1), filter_kind=params.filter_kind,
                           filter_params=tuple(params.filter_params))
        x0, x1, y0, y1 = _extent(rp)
        n = (x1 - x0 + 1) * (y1 - y0 + 1)
        return {"r2": np.full(n, np.float32(params.radius) * np.float32(params.radius), np.float32),
                "n": np.zeros(n, np.float32), "m": np.zeros(n, np.uint32)}

    def sppm_pass(self, params, width, height, pass_index=0, film=None, splats=None, state=None,
                  nthreads=0):
        """one SPPM pass; returns (film, splats, state, stats)"""
        if film is None:
            film = np.zeros((height, width, 4), np.float32)
        if splats is None:
            splats = np.zeros((height, width, 3), np.float32)
        if state is None:
            state = self.sppm_state(params, width, height)
        st = (C.c_uint64 * 4)()
        rc = lib().orc_sppm_pass(self.h, C.byref(params), width, height, pass_index, fp(film),
                                 fp(splats), fp(state["r2"]), fp(state["n"]),
                                 state["m"].ctypes.data_as(C.POINTER(C.c_uint32)),
                                 len(state["r2"]), nthreads, st)
        if rc != 0:
            raise ValueError(f"orc_sppm_pass failed: {rc}")
        return film, splats, state, {"rays_closest": st[0], "hitpoints": st[1], "splats": st[2],
                                     "nonfinite": st[3]}

    def texture(self, node, p, u=0.0, v=0.0):
        """texture node `node` at shading point p, surface (u, v): 16 bands
        for spectrum nodes, a float for scalar ones"""
        out = np.zeros(16, np.float32)
        pp = np.asarray(p, np.float32)
        rc = lib().orc_texture_eval(self.h, node, fp(pp), float(u), float(v), fp(out))
        if rc != 0:
            raise ValueError(f"orc_texture_eval failed: {rc}")
        return out if self.kinds[node] < abi.TEXN_SCALAR else np.float32(out[0])

    def sample_li(self, params, pass_index, px, py, n):
        xyz = np.zeros(3, np.float32)
        ras = np.zeros(2, np.float32)
        spec = np.zeros(16, np.float32)
        lib().orc_sample_li(self.h, C.byref(params), pass_index, px, py, n, fp(xyz), fp(ras), fp(spec))
        return xyz, ras, spec


def _extent(p):
    """imageWindow' (Image.hs:170-176) of render parameters"""
    import math
    if p.filter_kind == abi.FILTER_BOX:
        fw = fh = 0.5
    else:
        fw, fh = float(np.float32(p.filter_params[0])), float(np.float32(p.filter_params[1]))
    return (math.floor(np.float32(0.5) - np.float32(fw)),
            math.floor(np.float32(0.5) + np.float32(p.width) + np.float32(fw)),
            math.floor(np.float32(0.5) - np.float32(fh)),
            math.floor(np.float32(0.5) + np.float32(p.height) + np.float32(fh)))


def resolve(film):
    """film (w, X, Y, Z) -> linear sRGB (getPixel with no splats, Image.hs:302-315)."""
    from bling_gb300.spectrum import xyz_to_rgb
    w = film[..., 0]
    inv = np.where(w != 0, np.float32(1) / np.where(w != 0, w, 1), 0).astype(np.float32)
    r, g, b = xyz_to_rgb(film[..., 1] * inv, film[..., 2] * inv, film[..., 3] * inv)
    return np.stack([r, g, b], -1)
