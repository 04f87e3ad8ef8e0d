"""BVH construction on the GPU (BLING_FLAG_GPU_BVH: Morton order, PLOC
clustering, the binary node layout with one primitive per leaf).

The answers of ray queries do not depend on the tree (conservative boxes,
ties to the larger primitive ID), so a GPU-built scene must answer exactly as
the host-built one and as brute force (the trace tests run every parity case
on a GPU-built context too); renders must give the same films up to the order
of the film's float additions.  The tree's quality is checked by the work a
traversal does, against the host's binned-SAH tree."""
import time

import numpy as np
import pytest

from bling_gb300 import scene as S
from bling_gb300.api import Context
from oracle.oracle import OracleScene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gctx():
    ctx = Context(device=0, gpu_bvh=True)
    yield ctx
    ctx.close()


def test_1m_soup_same_answers_and_comparable_work(gpu_ctx, gctx):
    soup = S.triangle_soup(1 << 20, seed=1)
    g_host, g_gpu = gpu_ctx.scene(soup), gctx.scene(soup)
    st = g_gpu.stats()
    assert st["bvh_nodes"] == (1 << 20) - 1 and st["bvh_leaf_prims"] == 1 << 20
    rays = S.soup_rays(1 << 18, seed=2)
    t0, p0, b0 = g_host.closest(rays)
    t1, p1, b1 = g_gpu.closest(rays)
    assert np.array_equal(p0, p1)
    assert np.array_equal(t0.view(np.uint32), t1.view(np.uint32))
    assert np.array_equal(b0.view(np.uint32), b1.view(np.uint32))
    ra = S.soup_rays(1 << 18, seed=3, any_hit=True)
    assert np.array_equal(g_host.any(ra), g_gpu.any(ra))
    c_host, c_gpu = g_host.traversal_counts(rays), g_gpu.traversal_counts(rays)
    print("nodes/slots per ray: host SAH", c_host, "GPU PLOC", c_gpu)
    # one primitive per leaf: more inner nodes than the host's leaves of up
    # to four, fewer slot tests; the box tests must stay comparable
    assert c_gpu["nodes_per_ray"] <= 1.6 * c_host["nodes_per_ray"], (c_host, c_gpu)


def test_heightfield_builds_fast_and_renders_the_same(gpu_ctx, gctx):
    sc = S.heightfield_scene(ns=2048, n_spheres=4096, width=96, height=54, env_size=(64, 32))
    t0 = time.perf_counter()
    g_gpu = gctx.scene(sc)
    gpu_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    g_host = gpu_ctx.scene(sc)
    host_s = time.perf_counter() - t0
    sg, sh = g_gpu.stats(), g_host.stats()
    print(f"8.4M-triangle heightfield: BVH build {sg['bvh_build_ms']:.1f} ms on the GPU, "
          f"{sh['bvh_build_ms']:.1f} ms on the host; scene creation {gpu_s * 1e3:.0f} ms / "
          f"{host_s * 1e3:.0f} ms")
    assert gpu_s < host_s
    assert sg["bvh_build_ms"] < 0.1 * sh["bvh_build_ms"]
    p = S.heightfield_params(96, 54, spp_side=2, max_depth=8)
    fa, fb = gpu_ctx.film(96, 54), gctx.film(96, 54)
    g_host.render_pass(fa, p, 0)
    g_gpu.render_pass(fb, p, 0)
    a, b = fa.read(), fb.read()
    assert np.array_equal(a[..., 0], b[..., 0])
    scale = float(np.abs(a[..., 1:]).max()) + 1e-30
    assert np.allclose(a[..., 1:], b[..., 1:], rtol=1e-5, atol=1e-6 * scale)
    assert g_host.stats()["rays_closest"] == g_gpu.stats()["rays_closest"]


@pytest.mark.parametrize("n", [1, 2, 3, 37, 4097])
def test_small_scenes(gctx, n):
    """tiny scenes: a single primitive (one leaf, no inner node) and sizes
    around the radix sort's and the scan's block boundaries"""
    soup = S.triangle_soup(n, seed=n + 3)
    g, o = gctx.scene(soup), OracleScene(soup)
    rays = S.soup_rays(2048, seed=n)
    t, p, _ = g.closest(rays)
    to, po, _ = o.closest(rays, brute=True)
    assert np.array_equal(p, po)
    h = p >= 0
    assert np.array_equal(t[h].view(np.uint32), to[h].view(np.uint32))
    assert g.stats()["bvh_nodes"] == n - 1


def test_identical_centroids():
    """primitives whose boxes coincide (all Morton codes equal): the clustering
    still merges them all; answers follow the tie rule"""
    ctx = Context(device=0, gpu_bvh=True)
    try:
        rng = np.random.default_rng(5)
        c = rng.uniform(-1, 1, (64, 3))
        v = np.stack([c, c + [0.1, 0, 0], c + [0, 0.1, 0]], 1).reshape(-1, 3)
        v = np.concatenate([v] * 40)  # every triangle 40 times
        from bling_gb300 import abi
        from bling_gb300.spectrum import constant
        s = S.Scene()
        m = s.add_material(abi.MAT_MATTE, kd=constant(0.5))
        s.add_mesh(v, np.arange(len(v)), m)
        g, o = ctx.scene(s), OracleScene(s)
        rays = np.zeros((8, 1024), np.float32)
        tgt = c[rng.integers(0, 64, 1024)] + [0.02, 0.02, 0]
        rays[0:3] = (tgt + [0, 0, -3]).T
        rays[3:6] = np.array([0, 0, 1], np.float32)[:, None]
        rays[7] = np.inf
        t, p, _ = g.closest(rays)
        to, po, _ = o.closest(rays, brute=True)
        assert np.array_equal(p, po)
        assert (p[p >= 0] >= 64 * 39).all()  # the last copy wins
    finally:
        ctx.close()
