"""Scenes and rays shared by the ray-query tests (GPU parity and the
oracle's kd-tree tests): a height grid on integer planes, rays that run along
those planes with exact zero direction components, and a mix of triangles
and transformed analytic shapes."""
import numpy as np

from bling_gb300 import abi
from bling_gb300 import scene as S
from bling_gb300 import transform as xf
from bling_gb300.spectrum import constant


def _grid_scene(n=96, seed=4):
    """an n x n-cell height grid on integer x and z coordinates: its BVH boxes
    have faces on the integer planes"""
    rng = np.random.default_rng(seed)
    xs, zs = np.meshgrid(np.arange(n + 1, dtype=np.float32), np.arange(n + 1, dtype=np.float32))
    ys = rng.uniform(0.0, 0.5, xs.shape).astype(np.float32)
    v = np.stack([xs.ravel(), ys.ravel(), zs.ravel()], 1)
    idx = []
    for j in range(n):
        for i in range(n):
            a = j * (n + 1) + i
            idx += [a, a + 1, a + n + 2, a, a + n + 2, a + n + 1]
    sc = S.Scene()
    m = sc.add_material(abi.MAT_MATTE, kd=constant(0.5))
    sc.add_mesh(v, idx, m)
    sc.prim_order = [0]
    return sc


def _axis_plane_rays(n, count, seed, zero_axis):
    """rays whose direction has an exact zero (+0.0 or -0.0) on zero_axis and
    whose origin lies on an integer plane of that axis"""
    rng = np.random.default_rng(seed)
    o = np.stack([rng.integers(0, n + 1, count), np.full(count, 3.0),
                  rng.integers(0, n + 1, count)], 0).astype(np.float32)
    o[2 - zero_axis] += rng.uniform(0, 1, count).astype(np.float32)  # the other horizontal axis
    d = np.stack([rng.uniform(-1, 1, count), rng.uniform(-1, -0.05, count),
                  rng.uniform(-1, 1, count)], 0).astype(np.float32)
    d[zero_axis] = np.where(rng.uniform(size=count) < 0.5, np.float32(0.0), np.float32(-0.0))
    d /= np.linalg.norm(d, axis=0)
    d[zero_axis] = np.where(rng.uniform(size=count) < 0.5, np.float32(0.0), np.float32(-0.0))
    rays = np.concatenate([o, d, np.zeros((1, count), np.float32),
                           np.full((1, count), np.inf, np.float32)]).astype(np.float32)
    return np.ascontiguousarray(rays)


def _shape_scene(seed, n_tris=200, n_shapes=60):
    rng = np.random.default_rng(seed)
    s = S.Scene()
    m = s.add_material(abi.MAT_MATTE, kd=constant(0.5))
    c = rng.uniform(-1, 1, (n_tris, 3))
    v = np.stack([c, c + rng.normal(0, 0.2, (n_tris, 3)), c + rng.normal(0, 0.2, (n_tris, 3))], 1)
    s.add_mesh(v.reshape(-1, 3), np.arange(3 * n_tris), m)
    order = [0]
    kinds = [abi.SHAPE_SPHERE, abi.SHAPE_QUAD, abi.SHAPE_BOX, abi.SHAPE_DISK, abi.SHAPE_CYLINDER]
    for k in range(n_shapes):
        kind = kinds[k % 5]
        if kind == abi.SHAPE_SPHERE:
            prm = (rng.uniform(0.05, 0.3),)
        elif kind == abi.SHAPE_QUAD:
            prm = tuple(rng.uniform(0.05, 0.3, 2))
        elif kind == abi.SHAPE_BOX:
            lo = rng.uniform(-0.2, 0, 3)
            prm = tuple(lo) + tuple(lo + rng.uniform(0.05, 0.3, 3))
        elif kind == abi.SHAPE_DISK:
            prm = (rng.uniform(-0.1, 0.1), rng.uniform(0.1, 0.3), rng.uniform(0, 0.05),
                   rng.uniform(1, 2 * np.pi))
        else:
            prm = (rng.uniform(0.05, 0.2), -0.1, rng.uniform(0, 0.3), rng.uniform(1, 2 * np.pi))
        o2w = xf.rotate_x(rng.uniform(-180, 180)) @ xf.rotate_y(rng.uniform(-180, 180)) @ \
            xf.translate(*rng.uniform(-1, 1, 3))
        idx = s.add_shape(kind, prm, o2w, m)
        order.insert(int(rng.integers(0, len(order) + 1)), ~idx)
    s.prim_order = order
    return s
