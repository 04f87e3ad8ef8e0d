"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no golden vectors for this path: its only tests
(src/lib/Graphics/Bling/Main/Tests.hs:24-41) check that `rnd` lies in [0,1)
and that `shuffle` preserves the multiset.  The oracle is pinned here by
analytic answers (exact hit distances and barycentrics), by the reference's
own properties restated for the oracle's generator and permutation, by the
tie rule of the `nearest'` fold, and by bit-exact agreement of the binary32
restatements (transforms, spectra) with an independent host implementation.
"""
import math

import numpy as np
import pytest

from bling_gb300 import abi
from bling_gb300 import scene as S
from bling_gb300 import transform as xf
from bling_gb300.spectrum import constant, rgb_to_spectrum, spectrum_to_xyz, xyz_to_rgb
from oracle import oracle as O
from oracle.oracle import OracleScene

F = np.float32


def ray(o, d, tmin=0.0, tmax=np.inf):
    r = np.zeros((8, 1), np.float32)
    r[0:3, 0] = o
    r[3:6, 0] = d
    r[6, 0] = tmin
    r[7, 0] = tmax
    return r


def tri_scene(verts):
    s = S.Scene()
    m = s.add_material(abi.MAT_MATTE, kd=constant(0.5))
    v = np.asarray(verts, np.float32).reshape(-1, 3)
    s.add_mesh(v, np.arange(len(v)), m)
    return OracleScene(s)


def shape_scene(kind, params, o2w=None):
    s = S.Scene()
    m = s.add_material(abi.MAT_MATTE, kd=constant(0.5))
    s.add_shape(kind, params, o2w or xf.identity(), m)
    return OracleScene(s)


# ---------------------------------------------------------------- intersection KATs
def test_triangle_hit_exact():
    o = tri_scene([(0, 0, 0), (1, 0, 0), (0, 1, 0)])
    t, p, b = o.closest(ray((0.25, 0.25, -1), (0, 0, 1)), brute=True)
    assert p[0] == 0 and t[0] == 1.0 and tuple(b[0]) == (0.25, 0.25)


@pytest.mark.parametrize("o_,d,tmin,tmax,hit", [
    ((0.5, 0.5, -1), (0, 0, 1), 0, np.inf, True),      # on the hypotenuse b1 + b2 == 1
    ((0.0, 0.0, -1), (0, 0, 1), 0, np.inf, True),      # on a vertex
    ((0.6, 0.6, -1), (0, 0, 1), 0, np.inf, False),     # outside
    ((0.2, 0.2, -1), (1, 0, 0), 0, np.inf, False),     # parallel: divisor == 0
    ((0.2, 0.2, 1), (0, 0, 1), 0, np.inf, False),      # behind the origin
    ((0.2, 0.2, -1), (0, 0, 1), 0, 1.0, True),         # t == tmax is inclusive
    ((0.2, 0.2, -1), (0, 0, 1), 1.0, 2.0, True),       # t == tmin is inclusive
    ((0.2, 0.2, -1), (0, 0, 1), 0, 0.999, False),
])
def test_triangle_bounds(o_, d, tmin, tmax, hit):
    o = tri_scene([(0, 0, 0), (1, 0, 0), (0, 1, 0)])
    r = ray(o_, d, tmin, tmax)
    t, p, _ = o.closest(r, brute=True)
    assert (p[0] == 0) == hit
    assert bool(o.any(r, brute=True)[0]) == hit


@pytest.mark.parametrize("kind,params,o_,d,t_exp", [
    (abi.SHAPE_SPHERE, (1.0,), (0, 0, -3), (0, 0, 1), 2.0),
    (abi.SHAPE_SPHERE, (1.0,), (0, 0, 0), (0, 0, 1), 1.0),       # from inside: far root
    (abi.SHAPE_QUAD, (1.0, 1.0), (0.5, 0.5, -2), (0, 0, 1), 2.0),
    (abi.SHAPE_BOX, (-1, -1, -1, 1, 1, 1), (0, 0, -5), (0, 0, 1), 4.0),
    (abi.SHAPE_DISK, (0.0, 1.0, 0.0, 2 * math.pi), (0.5, 0, -1), (0, 0, 1), 1.0),
    (abi.SHAPE_CYLINDER, (1.0, -1.0, 1.0, 2 * math.pi), (-3, 0, 0), (1, 0, 0), 2.0),
])
def test_shape_hits_exact(kind, params, o_, d, t_exp):
    o = shape_scene(kind, params)
    t, p, _ = o.closest(ray(o_, d), brute=True)
    assert p[0] == 0 and t[0] == F(t_exp)


def test_shape_misses_and_partial_disk():
    o = shape_scene(abi.SHAPE_DISK, (0.0, 1.0, 0.0, math.pi / 2))
    assert o.closest(ray((0.5, 0.1, -1), (0, 0, 1)), brute=True)[1][0] == 0
    assert o.closest(ray((-0.5, 0.1, -1), (0, 0, 1)), brute=True)[1][0] == -1  # phi > phimax
    o = shape_scene(abi.SHAPE_QUAD, (1.0, 1.0))
    assert o.closest(ray((1.5, 0, -1), (0, 0, 1)), brute=True)[1][0] == -1


def test_transformed_sphere():
    o = shape_scene(abi.SHAPE_SPHERE, (0.5,), xf.translate(0, 0, 5))
    t, p, _ = o.closest(ray((0, 0, 0), (0, 0, 1)), brute=True)
    assert p[0] == 0 and t[0] == F(4.5)


def test_tie_goes_to_larger_primitive_id():
    v = [(0, 0, 0), (1, 0, 0), (0, 1, 0)]
    o = tri_scene(v * 3)
    t, p, _ = o.closest(ray((0.25, 0.25, -1), (0, 0, 1)), brute=True)
    assert p[0] == 2
    t2, p2, _ = o.closest(ray((0.25, 0.25, -1), (0, 0, 1)))
    assert p2[0] == 2


def test_oracle_bvh_equals_brute_force():
    soup = S.triangle_soup(20000, seed=3)
    o = OracleScene(soup)
    rays = S.soup_rays(3000, seed=4)
    tb, pb, bb = o.closest(rays, brute=True)
    tv, pv, bv = o.closest(rays)
    assert np.array_equal(pb, pv)
    h = pb >= 0
    assert np.array_equal(tb[h].view(np.uint32), tv[h].view(np.uint32))
    ra = S.soup_rays(3000, seed=5, any_hit=True)
    assert np.array_equal(o.any(ra, brute=True), o.any(ra))


# ---------------------------------------------------------------- the reference's properties
def test_rnd_in_unit_interval():
    """Tests.hs:24-29 -- rnd in [0, 1)"""
    out = np.empty(4096, np.float32)
    for k in range(8):
        O.lib().orc_random_floats(7, k, k, -k, 3, 0, 4096, O.fp(out))
        assert (out >= 0).all() and (out < 1).all()


@pytest.mark.parametrize("l", [1, 2, 3, 9, 16, 64, 100, 1000])
def test_permutation_preserves_multiset(l):
    """Tests.hs:31-41 -- shuffling preserves the multiset"""
    for p in (0, 1, 0xdeadbeef, 12345):
        perm = [O.lib().orc_permute(i, l, p) for i in range(l)]
        assert sorted(perm) == list(range(l))


# ---------------------------------------------------------------- spectra
def test_spectrum_tables_bit_exact_across_restatements():
    L = O.lib()
    for rgb in [(1, 1, 1), (0.63, 0.065, 0.05), (0.14, 0.45, 0.09), (0.2, 0.9, 0.4), (15, 15, 15)]:
        for illum in (0, 1):
            out = np.zeros(16, np.float32)
            L.orc_rgb_to_spectrum(illum, *map(float, rgb), O.fp(out))
            py = rgb_to_spectrum(rgb, bool(illum))
            assert np.array_equal(out.view(np.uint32), py.view(np.uint32))
            xyz = np.zeros(3, np.float32)
            L.orc_spectrum_to_xyz(O.fp(out), O.fp(xyz))
            assert np.array_equal(np.asarray(spectrum_to_xyz(py), np.float32).view(np.uint32),
                                  xyz.view(np.uint32))


def test_white_reflectance_is_flat_with_unit_luminance():
    """rgbToSpectrumRefl(1,1,1) is the white basis of the Smits tables (flat at
    about 1.062 over 400-700 nm); its XYZ is that of an equal-energy spectrum
    normalised by the banded sum of y-bar (Spectrum.hs:349-355) -- no
    white-point adaptation, so its sRGB is reddish (about 1.35, 1.07, 1.01)."""
    s = rgb_to_spectrum((1, 1, 1))
    assert np.allclose(s, s.mean(), rtol=0.005) and abs(s.mean() - 1.062) < 0.005
    x, y, z = spectrum_to_xyz(s)
    fx, fy, fz = spectrum_to_xyz(constant(1.0))
    assert abs(fy - 1) < 1e-6
    assert np.allclose(np.array([x, y, z]) / s.mean(), [fx, fy, fz], rtol=0.005)
    r, g, b = xyz_to_rgb(fx, fy, fz)
    assert abs(g - 0.95) < 0.05 and r > 1.15 and 0.85 < b < 1.0


# ---------------------------------------------------------------- transforms
def _oracle_xf(fn, *args):
    out = np.zeros(32, np.float32)
    fn(*args, O.fp(out))
    return out


def test_transforms_bit_exact():
    L = O.lib()
    cases = [
        (xf.translate(1.5, -2, 0.25), _oracle_xf(L.orc_xf_translate, 1.5, -2.0, 0.25)),
        (xf.scale(2, 3, 0.5), _oracle_xf(L.orc_xf_scale, 2.0, 3.0, 0.5)),
        (xf.rotate_x(-90), _oracle_xf(L.orc_xf_rotate, 0, -90.0)),
        (xf.rotate_y(18), _oracle_xf(L.orc_xf_rotate, 1, 18.0)),
        (xf.rotate_z(33.3), _oracle_xf(L.orc_xf_rotate, 2, 33.3)),
        (xf.perspective(40, 1e-2, 1000), _oracle_xf(L.orc_xf_perspective, 40.0, 1e-2, 1000.0)),
    ]
    pos, look, up = [np.asarray(v, np.float32) for v in ((0.5, 0.5, -1.4), (0.5, 0.5, 0.5), (0, 1, 0))]
    cases.append((xf.look_at(pos, look, up),
                  _oracle_xf(L.orc_xf_look_at, O.fp(pos), O.fp(look), O.fp(up))))
    a, b = xf.rotate_y(18), xf.translate(0.33, 0, 0.62)
    ab = np.zeros(32, np.float32)
    L.orc_xf_concat(O.fp(a.pack()), O.fp(b.pack()), O.fp(ab))
    cases.append((a @ b, ab))
    for t, ref in cases:
        assert np.array_equal(t.pack().view(np.uint32), ref.view(np.uint32))


def test_camera_bit_exact():
    c2w = xf.look_at((0.5, 0.5, -1.4), (0.5, 0.5, 0.5), (0, 1, 0))
    _, r2c = xf.perspective_camera(c2w, 0.0, 1.0, 40.0, 256, 192)
    cam = abi.CameraDesc()
    O.lib().orc_camera_perspective(O.fp(c2w.pack()), 0.0, 1.0, 40.0, 256.0, 192.0, cam)
    assert np.array_equal(np.asarray(cam.r2c[:], np.float32).view(np.uint32), r2c.m.view(np.uint32))
    assert np.array_equal(np.asarray(cam.r2c_inv[:], np.float32).view(np.uint32),
                          r2c.inv.view(np.uint32))


# ---------------------------------------------------------------- film
def test_box_filter_table_is_all_ones():
    out = np.zeros(256, np.float32)
    O.lib().orc_filter_table(abi.FILTER_BOX, O.fp(np.zeros(4, np.float32)), O.fp(out))
    assert (out == 1).all()


def test_mitchell_table_matches_formula():
    prm = np.asarray([2, 2, 1 / 3, 1 / 3], np.float32)
    out = np.zeros(256, np.float32)
    O.lib().orc_filter_table(abi.FILTER_MITCHELL, O.fp(prm), O.fp(out))
    B = C = 1 / 3

    def m1d(x):
        x = abs(2 * x)
        if x > 1:
            return ((-B - 6 * C) * x ** 3 + (6 * B + 30 * C) * x ** 2 + (-12 * B - 48 * C) * x
                    + (8 * B + 24 * C)) / 6
        return ((12 - 9 * B - 6 * C) * x ** 3 + (-18 + 12 * B + 6 * C) * x ** 2 + (6 - 2 * B)) / 6

    for y in range(16):
        for x in range(16):
            fx, fy = (x + 0.5) * 2 / 16, (y + 0.5) * 2 / 16
            assert abs(out[y * 16 + x] - m1d(fx / 2) * m1d(fy / 2)) < 1e-5


# ---------------------------------------------------------------- integrator
def _lit_plane(rho=0.5, cos_theta=0.6, strata=2, md=1):
    s = S.Scene()
    m = s.add_material(abi.MAT_MATTE, kd=constant(rho))
    v = np.array([[-10, 0, -10], [10, 0, -10], [10, 0, 10], [-10, 0, 10]], np.float32)
    s.add_mesh(v, [0, 1, 2, 0, 2, 3], m)
    sin_t = math.sqrt(1 - cos_theta ** 2)
    s.lights = [S.Light(abi.LIGHT_DIRECTIONAL, constant(2.0), vec=(sin_t, cos_theta, 0.0))]
    c2w = xf.look_at((0, 1, 0), (0, 0, 0.001), (0, 0, 1))
    c2w, r2c = xf.perspective_camera(c2w, 0.0, 1.0, 20.0, 8, 8)
    s.set_camera(c2w, r2c)
    p = S.render_params(8, 8, (strata, strata), max_depth=md, sample_depth=1, rr_depth=7)
    return s, p


def test_directional_light_on_lambertian_plane():
    """maxDepth 1: L = (rho/pi) cos(theta) * E |n.d| -- the reference applies the
    cosine twice for directional lights (Light.hs:143-145 and the Lambertian
    eval, Diffuse.hs:26)."""
    rho, ct, E = 0.5, 0.6, 2.0
    sc, p = _lit_plane(rho, ct)
    film, st = OracleScene(sc).render_pass(p, 0)
    w = film[..., 0]
    Y = film[..., 2] / np.where(w > 0, w, 1)
    L = rho / math.pi * ct * E * ct
    ys = spectrum_to_xyz(constant(L))[1]
    assert np.allclose(Y[w > 0], ys, rtol=2e-5)
    assert st["path_samples"] == 10 * 10 * 4


def test_cornell_oracle_render_is_deterministic_and_finite():
    sc = S.cornell_room(24, 24)
    p = S.cornell_params(24, 24, spp_side=2)
    o = OracleScene(sc)
    f1, s1 = o.render_pass(p, 0)
    f2, s2 = o.render_pass(p, 0)
    assert np.array_equal(f1, f2) and s1 == s2
    assert np.isfinite(f1).all()
    assert s1["path_samples"] == 26 * 26 * 4
    assert (f1[..., 0] > 0).all()
    y = f1[..., 2] / f1[..., 0]
    assert 0.05 < y.mean() < 2.0


def _furnace_ratio(film):
    """mean Y of the sphere's pixels over the mean Y of the background pixels"""
    w = film[..., 0]
    y = film[..., 2] / np.where(w > 0, w, 1)
    h, wd = y.shape
    yy, xx = np.mgrid[0:h, 0:wd]
    r = np.hypot(xx + 0.5 - wd / 2, yy + 0.5 - h / 2)
    inner = r < 0.25 * wd   # well inside the sphere's disc (radius ~0.39 of the width)
    outer = r > 0.48 * wd   # background corners
    return y[inner].mean() / y[outer].mean(), y[outer].mean()


def test_white_furnace_oracle():
    """A Lambertian sphere of albedo 0.5 under a uniform environment reflects
    exactly 0.5 of it (direct light only: reflected rays of a convex object
    escape, and a diffuse bounce adds no environment radiance afterwards)."""
    sc = S.furnace_scene(0.5, 24, 24)
    p = S.render_params(24, 24, (8, 8), max_depth=3, sample_depth=3, rr_depth=7)
    film, _ = OracleScene(sc).render_pass(p, 0)
    ratio, bg = _furnace_ratio(film)
    assert abs(ratio - 0.5) < 0.01, ratio
    assert abs(bg - spectrum_to_xyz(constant(1.0))[1]) < 1e-5


def _occupied_strata(o, params, px, py, side):
    """how many of the side x side pixel strata the pixel's samples fall in"""
    cells = set()
    for n in range(side * side):
        _, ras, _ = o.sample_li(params, 0, px, py, n)
        fx, fy = ras[0] - px, ras[1] - py
        assert 0.0 <= fx < 1.0 and 0.0 <= fy < 1.0
        cells.add((int(fx * side), int(fy * side)))
    return len(cells)


def test_random_sampler_is_not_stratified():
    """Stratified 8x8 puts one sample in each of the pixel's 64 strata;
    Random 64 (runSample (Random spp), Sampling.hs:101-110) draws the positions
    independently, which leaves strata empty (all 64 filled has probability
    64!/64^64)."""
    sc = S.cornell_room(8, 8)
    o = OracleScene(sc)
    strat = S.render_params(8, 8, (8, 8), max_depth=1)
    rand = S.render_params(8, 8, (64, 1), max_depth=1, sampler=abi.SAMPLER_RANDOM)
    for px, py in [(0, 0), (3, 5), (7, 7)]:
        assert _occupied_strata(o, strat, px, py, 8) == 64
        assert _occupied_strata(o, rand, px, py, 8) < 60


def test_random_sampler_converges_to_the_stratified_image():
    sc = S.cornell_room(16, 16)
    o = OracleScene(sc)
    fs, _ = o.render_pass(S.render_params(16, 16, (8, 8), max_depth=5, rr_depth=3), 0)
    fr, st = o.render_pass(S.render_params(16, 16, (64, 1), max_depth=5, rr_depth=3,
                                           sampler=abi.SAMPLER_RANDOM), 0)
    assert st["path_samples"] == 18 * 18 * 64
    assert np.array_equal(fs[..., 0], fr[..., 0])  # box filter: 64 samples per pixel on both
    ys, yr = fs[..., 2].sum() / fs[..., 0].sum(), fr[..., 2].sum() / fr[..., 0].sum()
    assert abs(yr - ys) < 0.03 * ys, (yr, ys)
