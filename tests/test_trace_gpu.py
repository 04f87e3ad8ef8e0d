"""Parity of the GPU ray queries with the CPU oracle (closest hit, any hit).

The oracle's answer is the reference's `nearest'` fold over all primitives in
primitive-ID order with the reference's intersection arithmetic: the smallest
t, ties to the larger primitive ID.  The GPU must reproduce it bit for bit:
same primitive, same t, same barycentrics.
"""
import numpy as np
import pytest

from bling_gb300 import abi
from bling_gb300 import scene as S
from bling_gb300 import transform as xf
from bling_gb300.api import BlingError
from bling_gb300.spectrum import constant
from oracle.oracle import OracleScene
from trace_cases import _axis_plane_rays, _grid_scene, _shape_scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wide_ctx():
    """A second context whose scenes use the 8-wide quantised BVH layout."""
    from bling_gb300.api import Context
    ctx = Context(device=0, wide_bvh=True)
    yield ctx
    ctx.close()


@pytest.fixture(scope="module")
def gpu_built_ctx():
    """A third context whose scenes build their BVH on the GPU."""
    from bling_gb300.api import Context
    ctx = Context(device=0, gpu_bvh=True)
    yield ctx
    ctx.close()


@pytest.fixture(scope="module")
def compact_ctx():
    """A fourth context whose scenes use 32-byte quantised binary nodes."""
    from bling_gb300.api import Context
    ctx = Context(device=0, compact_bvh=True)
    yield ctx
    ctx.close()


@pytest.fixture(params=["binary", "wide", "gpu-built", "compact"])
def ctx(request, gpu_ctx):
    """Every BVH layout, and the tree built on the GPU, must give the
    oracle's answers: traversal is conservative, so the answer does not
    depend on the tree."""
    if request.param == "binary":
        return gpu_ctx
    return request.getfixturevalue({"wide": "wide_ctx", "gpu-built": "gpu_built_ctx",
                                    "compact": "compact_ctx"}[request.param])


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def _check_closest(g, o, rays, brute=True):
    t, p, b = g.closest(rays)
    to, po, bo = o.closest(rays, brute=brute)
    assert np.array_equal(p, po), f"{np.count_nonzero(p != po)} primitive mismatches"
    h = p >= 0
    assert np.array_equal(_bits(t[h]), _bits(to[h]))
    assert np.array_equal(_bits(b[h]), _bits(bo[h]))
    assert np.all(np.isinf(t[~h]))
    return t, p


def test_soup_closest_and_any_vs_brute_force(ctx):
    soup = S.triangle_soup(30000, seed=5)
    g, o = ctx.scene(soup), OracleScene(soup)
    rays = S.soup_rays(4096, seed=6)
    t, p = _check_closest(g, o, rays)
    assert 0.3 < (p >= 0).mean() < 1.0
    ra = S.soup_rays(4096, seed=7, any_hit=True)
    assert np.array_equal(g.any(ra), o.any(ra, brute=True))


def test_1m_soup_vs_oracle_bvh(ctx):
    soup = S.triangle_soup(1 << 20, seed=1)
    g, o = ctx.scene(soup), OracleScene(soup)
    rays = S.soup_rays(1 << 17, seed=2)
    _check_closest(g, o, rays, brute=False)
    ra = S.soup_rays(1 << 17, seed=3, any_hit=True)
    assert np.array_equal(g.any(ra), o.any(ra))
    # a brute-force spot check at full scene size
    sub = np.ascontiguousarray(rays[:, :512])
    _check_closest(g, o, sub, brute=True)


@pytest.mark.parametrize("zero_axis", [0, 2])
def test_zero_direction_component_on_box_faces(ctx, zero_axis):
    """rays with a zero direction component that run along BVH box faces (0 *
    inf in the slab test): same answers as brute force, and no more traversal
    work than rays tilted off the plane (binary layout; the 8-wide layout
    ignores the zero axis in the box test, which is conservative but visits
    more nodes)"""
    n = 96
    sc = _grid_scene(n)
    g, o = ctx.scene(sc), OracleScene(sc)
    rays = _axis_plane_rays(n, 4096, 8 + zero_axis, zero_axis)
    t, p = _check_closest(g, o, rays)
    assert (p >= 0).mean() > 0.5
    ra = rays.copy()
    ra[7] = np.where(p >= 0, t, 5.0)  # any hit up to the closest hit
    assert np.array_equal(g.any(ra), o.any(ra, brute=True))
    if not ctx.wide_bvh:
        tilted = rays.copy()
        tilted[3 + zero_axis] = 1e-3
        c0, c1 = g.traversal_counts(rays), g.traversal_counts(tilted)
        assert c0["nodes_per_ray"] <= 3 * c1["nodes_per_ray"], (c0, c1)


def test_1m_soup_vs_reference_kdtree(gpu_ctx):
    """The GPU against the reference's own acceleration structure (the
    oracle's kd-tree restatement, Primitive/KdTree.hs): the same primitive
    except at ties, where the kd-tree keeps the equal-distance hit its leaf
    order tests last; the distance bit-identical for every ray."""
    soup = S.triangle_soup(1 << 20, seed=1)
    g, o = gpu_ctx.scene(soup), OracleScene(soup)
    rays = S.soup_rays(1 << 17, seed=2)
    t, p, b = g.closest(rays)
    tk, pk, bk, _ = o.closest_kd(rays)
    assert np.array_equal(p >= 0, pk >= 0)
    h = p >= 0
    assert np.array_equal(_bits(t[h]), _bits(tk[h]))
    ties = np.nonzero(p != pk)[0]
    assert len(ties) <= 1e-4 * len(p), ties  # ties are rare in a random soup
    same = h & (p == pk)
    assert np.array_equal(_bits(b[same]), _bits(bk[same]))
    ra = S.soup_rays(1 << 17, seed=3, any_hit=True)
    hk, _ = o.any_kd(ra)
    assert np.array_equal(g.any(ra), hk)


def test_host_buffer_chunks_equal_device_buffer_queries(gpu_ctx):
    """the host-buffer calls copy, trace and copy back in chunks of 2^21 rays
    on three streams; a ragged count over several chunks gives exactly the
    device-buffer answers"""
    import torch
    soup = S.triangle_soup(1 << 18, seed=9)
    g = gpu_ctx.scene(soup)
    n = (1 << 22) + 12345
    rays = S.soup_rays(n, seed=10)
    t, p, b = g.closest(rays)
    dev = torch.device("cuda", 0)
    d_r = torch.from_numpy(rays).to(dev)
    d_t = torch.empty(n, dtype=torch.float32, device=dev)
    d_p = torch.empty(n, dtype=torch.int32, device=dev)
    d_b = torch.empty(2 * n, dtype=torch.float32, device=dev)
    g.closest_device(d_r, d_t, d_p, d_b)
    torch.cuda.synchronize()
    assert np.array_equal(p, d_p.cpu().numpy())
    assert np.array_equal(_bits(t), _bits(d_t.cpu().numpy()))
    assert np.array_equal(_bits(b.ravel()), _bits(d_b.cpu().numpy()))
    ra = S.soup_rays(n, seed=11, any_hit=True)
    h = g.any(ra)
    d_h = torch.empty(n, dtype=torch.uint8, device=dev)
    g.any_device(torch.from_numpy(ra).to(dev), d_h)
    torch.cuda.synchronize()
    assert np.array_equal(h, d_h.cpu().numpy())
    assert 0.05 < h.mean() < 0.999


def test_full_size_closest_is_closest(gpu_ctx):
    """16M rays over the 1M soup: any-hit with tmax just below the reported
    closest t finds nothing, with tmax = t finds the hit."""
    soup = S.triangle_soup(1 << 20, seed=1)
    g = gpu_ctx.scene(soup)
    rays = S.soup_rays(1 << 24, seed=2)
    t, p, _ = g.closest(rays, with_bary=False)
    h = p >= 0
    assert h.mean() > 0.5
    below = rays.copy()
    below[7] = np.where(h, np.nextafter(t, np.float32(0)), np.inf)
    assert not g.any(below)[h].any()
    at = rays.copy()
    at[7] = np.where(h, t, np.inf)
    any_at = g.any(at)
    assert any_at[h].all() and not any_at[~h].any()


@pytest.mark.parametrize("seed", [21, 22])
def test_analytic_shapes_vs_brute_force(ctx, seed):
    sc = _shape_scene(seed)
    g, o = ctx.scene(sc), OracleScene(sc)
    rays = S.soup_rays(8192, seed=seed + 100)
    rays[0:3] *= 0.7  # some origins inside shapes
    _check_closest(g, o, rays)
    ra = S.soup_rays(8192, seed=seed + 200, any_hit=True)
    assert np.array_equal(g.any(ra), o.any(ra, brute=True))


def test_ties_go_to_the_larger_primitive_id(ctx):
    rng = np.random.default_rng(3)
    c = rng.uniform(-1, 1, (500, 3))
    v = np.stack([c, c + [0.1, 0, 0], c + [0, 0.1, 0]], 1).reshape(-1, 3)
    v = np.concatenate([v, v, v])  # every triangle three times
    s = S.Scene()
    m = s.add_material(abi.MAT_MATTE, kd=constant(0.5))
    s.add_mesh(v, np.arange(len(v)), m)
    g, o = ctx.scene(s), OracleScene(s)
    rays = np.zeros((8, 4096), np.float32)
    tgt = c[rng.integers(0, 500, 4096)] + [0.02, 0.02, 0]
    rays[0:3] = (tgt + [0, 0, -3]).T
    rays[3:6] = np.array([0, 0, 1], np.float32)[:, None]
    rays[7] = np.inf
    t, p = _check_closest(g, o, rays)
    assert (p[p >= 0] >= 1000).all()  # the third copy wins


def test_edge_cases(ctx):
    soup = S.triangle_soup(5000, seed=8)
    g, o = ctx.scene(soup), OracleScene(soup)
    empty = np.zeros((8, 0), np.float32)
    t, p, _ = g.closest(empty)
    assert t.size == 0 and g.any(empty).size == 0
    rng = np.random.default_rng(9)
    rays = np.zeros((8, 3000), np.float32)
    rays[0:3] = rng.uniform(-1.2, 1.2, (3, 3000))
    d = np.zeros((3, 3000), np.float32)
    axis = rng.integers(0, 3, 3000)
    d[axis, np.arange(3000)] = rng.choice([-1.0, 1.0], 3000)  # axis-aligned: two zero components
    rays[3:6] = d
    rays[6] = rng.choice([0.0, 0.5], 3000)
    rays[7] = rng.choice([np.inf, 0.3, 0.0], 3000)  # includes tmin > tmax
    _check_closest(g, o, rays)
    assert np.array_equal(g.any(rays), o.any(rays, brute=True))


def test_nan_rays_are_degenerate_and_cheap(ctx):
    soup = S.triangle_soup(1 << 20, seed=1)
    g = ctx.scene(soup)
    rays = S.soup_rays(4096, seed=4)
    rays[3, ::7] = np.nan  # NaN direction component
    rays[0, 3::11] = np.nan  # NaN origin component
    bad = np.isnan(rays).any(0)
    t, p, _ = g.closest(rays)
    assert (p[bad] == -2).all() and np.isnan(t[bad]).all()
    assert (p[~bad] != -2).all()
    assert g.any(rays)[bad].all()
    # the good rays still get the oracle's answers
    o = OracleScene(soup)
    good = np.ascontiguousarray(rays[:, ~bad][:, :512])
    _check_closest(g, o, good, brute=False)


@pytest.mark.parametrize("bad", ["negative", "not_multiple_of_3", "out_of_range"])
def test_mesh_validation(gpu_ctx, bad):
    s = S.Scene()
    m = s.add_material(abi.MAT_MATTE, kd=constant(0.5))
    v = np.zeros((4, 3), np.float32)
    idx = {"negative": [0, 1, -1], "not_multiple_of_3": [0, 1, 2, 3],
           "out_of_range": [0, 1, 4]}[bad]
    s.add_mesh(v, idx, m)
    with pytest.raises(BlingError) as e:
        gpu_ctx.scene(s)
    assert e.value.code == abi.BLING_ERR_INVALID_ARG


def test_unknown_material_kind_is_refused(gpu_ctx):
    s = S.Scene()
    m = s.add_material(abi.MAT_MATTE, kd=constant(0.5))
    s.materials[m].kind = 9
    s.add_shape(abi.SHAPE_SPHERE, (1.0,), xf.identity(), m)
    with pytest.raises(BlingError) as e:
        gpu_ctx.scene(s)
    assert e.value.code == abi.BLING_ERR_INVALID_ARG and "unknown kind" in str(e.value)
