"""The oracle's restatement of the reference's kd-tree (Primitive/KdTree.hs),
checked on the CPU.

The reference finds the closest hit by walking its kd-tree front to back and
folding `nearest'` over each leaf, so among hits at the same distance the one
tested last wins, and the order depends on the tree.  Brute force in
primitive-ID order (the oracle's golden rule, which the GPU reproduces) gives
the larger primitive ID.  The two may therefore differ only at ties: the
kd-tree's primitive must hit at the very same distance.  Any-hit answers test
the whole ray interval in every leaf, so they must agree exactly.

One more difference is the reference's own: its root slab test
(intersectAABB, AABB.hs:79-94) computes 1 / d, so a ray with a zero
direction component whose origin lies exactly on the scene box's face on
that axis gets 0 * inf = NaN for one slab distance and +-inf for the other;
with GHC's max/min that empties the interval for -0.0 on the low face (and
for either sign on the high face, after the other slabs), and the reference
misses every hit of such a ray.  Those rays are flagged, not failed: the test
checks that each non-tie difference is such a ray.

The build is checked against the reference's rules: depth limit
round(8 + 3 ln N) (GHC's `round`: halves to even), every interior node
splits its cell strictly inside, and the tree holds every primitive.
"""
import math

import numpy as np
import pytest

from bling_gb300 import scene as S
from oracle.oracle import OracleScene
from trace_cases import _axis_plane_rays, _grid_scene, _shape_scene


def _scene_box(sc):
    """the scene's world bounds over its mesh vertices (triangle scenes)"""
    v = np.concatenate([m.vertices for m in sc.meshes])
    return v.min(0), v.max(0)


def _on_box_face_with_zero_dir(rays, lo, hi):
    """rays with a zero direction component whose origin lies on the scene
    box's face on that axis"""
    o, d = rays[0:3], rays[3:6]
    f = np.zeros(rays.shape[1], bool)
    for a in range(3):
        f |= (d[a] == 0) & ((o[a] == lo[a]) | (o[a] == hi[a]))
    return f


def _flag(rays, tb, pb, tk, pk, box=None):
    """rays where the kd-tree and brute force differ: ties (same distance,
    another primitive) and, given the scene box, the root-slab misses of rays
    on its faces.  Asserts there is nothing else; returns (ties, slab)."""
    slab = np.zeros(len(pb), bool)
    if box is not None:
        slab = _on_box_face_with_zero_dir(rays, *box) & (pb >= 0) & (pk < 0)
    rest = ~slab
    h = (pb >= 0) & rest
    assert np.array_equal((pb >= 0)[rest], (pk >= 0)[rest])
    assert np.array_equal(tb[h].view(np.uint32), tk[h].view(np.uint32))
    ties = np.nonzero(rest & (pb != pk))[0]
    return ties, np.nonzero(slab)[0]


def _ties_only(o, rays, tb, pb, tk, pk):
    ties, _ = _flag(rays, tb, pb, tk, pk)
    return ties


def test_depth_limit_and_structure():
    for n in (1, 2, 7, 100, 4096):
        soup = S.triangle_soup(n, seed=n)
        st = OracleScene(soup).kdtree()
        md = np.float32(8) + np.float32(3) * np.log(np.float32(n))
        assert st["depth_limit"] == int(np.rint(md))  # rint: halves to even, as GHC's round
        assert st["max_depth"] <= st["depth_limit"]
        assert st["leaves"] == st["interiors"] + 1
        assert st["leaf_refs"] >= n  # every primitive in at least one leaf
    assert OracleScene(S.triangle_soup(1, seed=1)).kdtree()["interiors"] == 0
    # round(8 + 3 ln N) at N = 4096 is 33 (8 + 24.95)
    assert int(np.rint(np.float32(8) + np.float32(3) * np.log(np.float32(4096)))) == 33
    assert math.isclose(8 + 3 * math.log(4096), 32.95, abs_tol=0.01)


def test_soup_kd_vs_brute_force():
    soup = S.triangle_soup(30000, seed=5)
    o = OracleScene(soup)
    rays = S.soup_rays(20000, seed=6)
    tb, pb, bb = o.closest(rays, brute=True)
    tk, pk, bk, cnt = o.closest_kd(rays)
    ties = _ties_only(o, rays, tb, pb, tk, pk)
    assert len(ties) <= 2, ties
    same = pb == pk
    assert np.array_equal(bb[same].view(np.uint32), bk[same].view(np.uint32))
    assert 0.3 < (pb >= 0).mean() < 1.0
    assert cnt["nodes"] > 0 and cnt["prims"] > 0
    ra = S.soup_rays(20000, seed=7, any_hit=True)
    hk, _ = o.any_kd(ra)
    assert np.array_equal(hk, o.any(ra, brute=True))


def test_ties_are_resolved_by_leaf_order():
    """three copies of every triangle: brute force picks the last copy (the
    largest ID); the kd-tree picks the copy its leaf tests last, at the same
    distance -- a tie, flagged rather than an error"""
    rng = np.random.default_rng(3)
    c = rng.uniform(-1, 1, (500, 3))
    v = np.stack([c, c + [0.1, 0, 0], c + [0, 0.1, 0]], 1).reshape(-1, 3)
    v = np.concatenate([v, v, v])
    from bling_gb300 import abi
    from bling_gb300.spectrum import constant
    s = S.Scene()
    m = s.add_material(abi.MAT_MATTE, kd=constant(0.5))
    s.add_mesh(v, np.arange(len(v)), m)
    o = OracleScene(s)
    rays = np.zeros((8, 4096), np.float32)
    tgt = c[rng.integers(0, 500, 4096)] + [0.02, 0.02, 0]
    rays[0:3] = (tgt + [0, 0, -3]).T
    rays[3:6] = np.array([0, 0, 1], np.float32)[:, None]
    rays[7] = np.inf
    tb, pb, _ = o.closest(rays, brute=True)
    tk, pk, _, _ = o.closest_kd(rays)
    _ties_only(o, rays, tb, pb, tk, pk)
    h = pb >= 0
    assert (pb[h] >= 1000).all()
    assert np.array_equal(pk[h] % 500, pb[h] % 500)  # the same triangle, some copy


@pytest.mark.parametrize("zero_axis", [0, 2])
def test_rays_along_split_planes(zero_axis):
    """a grid whose triangle bounds (so the kd-tree's split planes) lie on
    integer planes, queried by rays with exact zero direction components
    running along those planes: tp = (split - o) * inf is NaN or infinite"""
    n = 48
    sc = _grid_scene(n)
    o = OracleScene(sc)
    rays = _axis_plane_rays(n, 4096, 8 + zero_axis, zero_axis)
    tb, pb, _ = o.closest(rays, brute=True)
    tk, pk, _, _ = o.closest_kd(rays)
    box = _scene_box(sc)
    ties, slab = _flag(rays, tb, pb, tk, pk, box)
    # the grid's x and z range is [0, n]: the rays whose origin is on x (or
    # z) = 0 or n with a zero direction there are the reference's misses
    edge = _on_box_face_with_zero_dir(rays, *box)
    assert len(slab) > 0 and set(slab) <= set(np.nonzero(edge)[0])
    ra = rays.copy()
    ra[7] = np.where(pb >= 0, tb, 5.0)
    hk, _ = o.any_kd(ra)
    hb = o.any(ra, brute=True)
    differ = np.nonzero(hk != hb)[0]
    assert set(differ) <= set(np.nonzero(edge)[0]), differ
    # off the box faces the two agree exactly
    assert np.array_equal(hk[~edge], hb[~edge])


@pytest.mark.parametrize("seed", [21, 22])
def test_analytic_shapes_kd_vs_brute_force(seed):
    sc = _shape_scene(seed)
    o = OracleScene(sc)
    rays = S.soup_rays(8192, seed=seed + 100)
    rays[0:3] *= 0.7
    tb, pb, _ = o.closest(rays, brute=True)
    tk, pk, _, _ = o.closest_kd(rays)
    _ties_only(o, rays, tb, pb, tk, pk)
    ra = S.soup_rays(8192, seed=seed + 200, any_hit=True)
    hk, _ = o.any_kd(ra)
    assert np.array_equal(hk, o.any(ra, brute=True))


def test_renders_through_the_kd_tree_match():
    """the oracle's path integrator gives the same film through the kd-tree
    as through its BVH (same random numbers): only tie rays could differ"""
    sc = S.cornell_room(40, 40)
    p = S.cornell_params(40, 40, spp_side=2, max_depth=5, rr_depth=3)
    o = OracleScene(sc)
    fb, sb = o.render_pass(p, 0)
    o.use_kdtree(True)
    fk, sk = o.render_pass(p, 0)
    assert sb == sk
    assert np.array_equal(fb, fk)
