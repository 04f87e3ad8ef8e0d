"""The host BVH builder on CPU (no GPU): structure of the binary and the
quantised 8-wide layouts for small, degenerate and large primitive sets."""
import ctypes as C

import numpy as np
import pytest

from bling_gb300 import build as gbuild
from bling_gb300 import scene as S


@pytest.fixture(scope="module")
def so():
    L = C.CDLL(str(gbuild.build()))
    L.bling_bvh_selftest.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int64,
                                     C.c_int32, C.POINTER(C.c_int64)]
    L.bling_bvh_selftest.restype = C.c_int
    return L


def selftest(so, lo, hi, max_leaf=4):
    lo = np.ascontiguousarray(lo, np.float32)
    hi = np.ascontiguousarray(hi, np.float32)
    st = (C.c_int64 * 5)()
    rc = so.bling_bvh_selftest(lo.ctypes.data_as(C.POINTER(C.c_float)),
                               hi.ctypes.data_as(C.POINTER(C.c_float)), len(lo), max_leaf, st)
    return rc, list(st)


@pytest.mark.parametrize("n", [1, 2, 3, 7, 8, 9, 17, 100, 1000])
def test_small_random_sets(so, n):
    rng = np.random.default_rng(n)
    c = rng.uniform(-1, 1, (n, 3))
    e = rng.uniform(0, 0.2, (n, 3))
    rc, st = selftest(so, c - e, c + e)
    assert rc == 0, (rc, st)


def test_coincident_and_flat_boxes(so):
    n = 300
    lo = np.zeros((n, 3), np.float32)
    hi = np.zeros((n, 3), np.float32)
    hi[:, 0] = 1.0  # flat in y and z, all centroids equal
    rc, st = selftest(so, lo, hi)
    assert rc == 0, (rc, st)


def test_soup_and_heightfield_layouts(so):
    soup = S.triangle_soup(200000, seed=2)
    v = soup.meshes[0].vertices.reshape(-1, 3, 3)
    rc, st = selftest(so, v.min(1), v.max(1))
    assert rc == 0 and st[1] > 0, (rc, st)  # the wide layout is built
    hf = S.heightfield_scene(ns=257, n_spheres=0, width=8, height=8, env_size=(8, 4))
    m = hf.meshes[0]
    tri = m.vertices[m.indices.reshape(-1, 3)]
    rc, st = selftest(so, tri.min(1), tri.max(1))
    assert rc == 0 and st[1] > 0, (rc, st)


@pytest.mark.parametrize("leaf", [1, 2, 3, 6, 8])
def test_leaf_sizes(so, leaf):
    rng = np.random.default_rng(leaf)
    c = rng.uniform(-5, 5, (5000, 3))
    rc, st = selftest(so, c - 0.01, c + 0.01, leaf)
    assert rc == 0, (rc, st)
