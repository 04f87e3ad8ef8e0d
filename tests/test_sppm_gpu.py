"""Parity of the GPU SPPM pass (bling_sppm_pass) with the CPU oracle.

Both sides draw the same random numbers for the camera trees and the
photons and build the same spatial hash (same cells, same bucket function,
same bucket membership), so every photon finds the same hit points.  The
camera samples' film weights are identical (box filter); XYZ, splats and
radii agree to float rounding except where a transcendental (sinf/cosf/powf)
perturbation sends a path elsewhere: at least 97% of pixels within 1e-3
relative (90% within 2e-3 with glass), means within 0.5%, hit-point counts
equal, splat counts within 1%.
"""
import numpy as np
import pytest

from bling_gb300 import abi, image
from bling_gb300 import scene as S
from bling_gb300 import transform as xf
from bling_gb300.spectrum import constant, rgb_to_spectrum
from oracle.oracle import OracleScene

pytestmark = pytest.mark.gpu

F = np.float32


def _both(gpu_ctx, sc, w, h, sp, passes=1):
    g = gpu_ctx.scene(sc)
    film = gpu_ctx.film(w, h)
    o = OracleScene(sc)
    f = spl = st = None
    sts = []
    for k in range(passes):
        g.sppm_pass(film, sp, k)
        f, spl, st, s = o.sppm_pass(sp, w, h, k, f, spl, st)
        sts.append(s)
    return film, g, (f, spl, st), sts


def _close(a, b, rel, frac):
    scale = np.abs(b).mean() + 1e-12
    err = np.abs(a - b) / (np.abs(b) + 1e-3 * scale)
    close = (err <= rel).all(-1) if a.ndim == 3 else err <= rel
    assert close.mean() >= frac, f"only {close.mean():.4f} within {rel}"
    ma, mb = a.mean(axis=tuple(range(a.ndim - 1))), b.mean(axis=tuple(range(b.ndim - 1)))
    assert np.all(np.abs(ma - mb) <= 5e-3 * np.abs(mb) + 1e-9), (ma, mb)


def _check(film, g, ref, sts, rel=1e-3, frac=0.97):
    f, spl, st = ref
    fg = film.read()
    assert np.array_equal(fg[..., 0], f[..., 0]), "camera-sample weights differ"
    _close(fg[..., 1:], f[..., 1:], rel, frac)
    _close(film.read_splats(), spl, rel, frac)
    r2 = film.read_sppm_radii()
    assert r2.shape == st["r2"].shape
    assert np.mean(np.abs(r2 - st["r2"]) <= 1e-5 * st["r2"]) >= frac
    gs = g.stats()
    assert abs(gs["light_splats"] - sum(s["splats"] for s in sts)) <= 0.01 * sum(s["splats"] for s in sts) + 2
    assert gs["nonfinite_drops"] == 0


def test_cornell_room_sppm_vs_oracle(gpu_ctx):
    sc = S.cornell_room(40, 40)
    sp = abi.sppm_params(100_000, max_depth=4, radius=0.02, alpha=0.7, seed=5)
    film, g, ref, sts = _both(gpu_ctx, sc, 40, 40, sp, passes=3)
    _check(film, g, ref, sts)


def _glass_scene(w=40, h=40):
    s = S.Scene()
    wall = s.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum((0.7, 0.7, 0.7)))
    plastic = s.add_material(abi.MAT_PLASTIC, kd=rgb_to_spectrum((0.2, 0.3, 0.7)),
                             ks=constant(0.4), roughness=0.1)
    glass = s.add_material(abi.MAT_GLASS, ks=constant(1.0), kt=constant(1.0), ior=1.5)
    mirror = s.add_material(abi.MAT_MIRROR, ks=rgb_to_spectrum((0.9, 0.9, 0.8)))
    v = np.array([[-3, -3, 2], [3, -3, 2], [3, 3, 2], [-3, 3, 2]], np.float32)
    s.add_mesh(v, [0, 1, 2, 0, 2, 3], wall)
    order = [0]
    order.append(~s.add_shape(abi.SHAPE_SPHERE, (0.7,), xf.translate(-0.5, 0, 0), glass))
    order.append(~s.add_shape(abi.SHAPE_SPHERE, (0.4,), xf.translate(0.9, -0.4, 0.5), mirror))
    order.append(~s.add_shape(abi.SHAPE_SPHERE, (0.4,), xf.translate(0.9, 0.6, 0.8), plastic))
    order.append(~s.add_shape(abi.SHAPE_SPHERE, (0.3,), xf.translate(0, 2, -1), wall,
                              emission=rgb_to_spectrum((6, 6, 6), illuminant=True)))
    s.prim_order = order
    s.lights = [S.Light(abi.LIGHT_POINT, rgb_to_spectrum((1, 1, 1), illuminant=True),
                        vec=(1.5, 1.5, -1.5))]
    s.set_perspective(xf.look_at((0, 0, -4), (0, 0, 0), (0, 1, 0)), 0.0, 1.0, 40.0, w, h)
    return s


def test_specular_branching_and_materials_vs_oracle(gpu_ctx):
    sc = _glass_scene()
    sp = abi.sppm_params(100_000, max_depth=6, radius=0.05, alpha=0.7, seed=2,
                         filter_kind=abi.FILTER_MITCHELL, filter_params=(2, 2, 1 / 3, 1 / 3))
    film, g, ref, sts = _both(gpu_ctx, sc, 40, 40, sp, passes=2)
    f, spl, st = ref
    fg = film.read()
    assert np.allclose(fg[..., 0], f[..., 0], rtol=1e-5, atol=1e-6)
    _close(fg[..., 1:], f[..., 1:], 2e-3, 0.9)
    _close(film.read_splats(), spl, 2e-3, 0.9)
    assert sts[0]["hitpoints"] > 0


def test_sunsky_sppm_vs_oracle(gpu_ctx):
    from test_sunsky import sunsky_scene
    sc = sunsky_scene(40, 30)
    sp = abi.sppm_params(100_000, max_depth=4, radius=0.1, alpha=0.7, seed=9)
    film, g, ref, sts = _both(gpu_ctx, sc, 40, 30, sp, passes=2)
    _check(film, g, ref, sts, rel=2e-3, frac=0.9)


def test_sppm_converges_to_the_path_tracer(gpu_ctx):
    W = H = 48
    sc = S.cornell_room(W, H)
    g = gpu_ctx.scene(sc)
    ptf = gpu_ctx.film(W, H)
    g.render_pass(ptf, S.cornell_params(W, H, spp_side=24, max_depth=40, rr_depth=3), 0)
    pt = ptf.resolve()
    film = gpu_ctx.film(W, H)
    n, passes = 1_000_000, 16
    sp = abi.sppm_params(n, max_depth=5, radius=0.015, alpha=0.7, seed=9)
    for k in range(passes):
        g.sppm_pass(film, sp, k)
    sn = int(np.ceil(np.sqrt(F(n))))
    img = film.resolve_splats(1.0 / (passes * sn * sn))
    for sl in (np.s_[18:30, 18:30], np.s_[38:46, 12:36], np.s_[12:24, 12:36], np.s_[16:32, 2:8]):
        a, b = pt[sl].mean((0, 1)), img[sl].mean((0, 1))
        assert np.all(np.abs(a - b) <= 0.05 * np.abs(a) + 1e-3), (sl, a, b)


def test_clear_resets_the_radii(gpu_ctx):
    sc = S.cornell_room(16, 16)
    g = gpu_ctx.scene(sc)
    film = gpu_ctx.film(16, 16)
    assert film.read_sppm_radii().size == 0
    sp = abi.sppm_params(10_000, max_depth=3, radius=0.03, alpha=0.5)
    g.sppm_pass(film, sp, 0)
    r = film.read_sppm_radii()
    assert r.size == 18 * 18 and (r < F(0.03) * F(0.03)).any()
    film.clear()
    assert film.read_sppm_radii().size == 0 and not film.read_splats().any()


def test_invalid_parameters_are_refused(gpu_ctx):
    sc = S.cornell_room(16, 16)
    g = gpu_ctx.scene(sc)
    film = gpu_ctx.film(16, 16)
    for kw in ({"alpha": 1.0}, {"radius": 0.0}, {"max_depth": 0}, {"max_depth": 25}):
        args = dict(photons=1000, max_depth=3, radius=0.03, alpha=0.5)
        args.update(kw)
        with pytest.raises(Exception):
            g.sppm_pass(film, abi.sppm_params(**args), 0)


def test_edge_cases_no_lights_no_hit_points(gpu_ctx):
    """a scene without lights: the light tracer and SPPM add nothing; a view
    of empty space: SPPM records no hit points and skips its photon pass;
    zero photons: ceil(sqrt 0) = 0 is raised to one photon (SPPM.hs:474)"""
    s = S.Scene()
    m = s.add_material(abi.MAT_MATTE, kd=constant(0.5))
    s.add_shape(abi.SHAPE_SPHERE, (1.0,), xf.identity(), m)
    s.set_perspective(xf.look_at((0, 0, -4), (0, 0, 0), (0, 1, 0)), 0.0, 1.0, 40.0, 16, 16)
    g = gpu_ctx.scene(s)
    film = gpu_ctx.film(16, 16)
    g.light_pass(film, 10_000)
    g.sppm_pass(film, abi.sppm_params(10_000, max_depth=3, radius=0.05, alpha=0.7), 0)
    assert not film.read_splats().any()
    o = OracleScene(s)
    _, spl, _, st = o.sppm_pass(abi.sppm_params(10_000, max_depth=3, radius=0.05, alpha=0.7), 16, 16)
    assert not spl.any() and st["splats"] == 0
    # looking away from everything: no hit points
    s.lights = [S.Light(abi.LIGHT_POINT, constant(1.0), vec=(0.0, 3.0, 0.0))]
    s.set_perspective(xf.look_at((0, 0, -4), (0, 0, -8), (0, 1, 0)), 0.0, 1.0, 40.0, 16, 16)
    g2 = gpu_ctx.scene(s)
    f2 = gpu_ctx.film(16, 16)
    g2.sppm_pass(f2, abi.sppm_params(0, max_depth=3, radius=0.05, alpha=0.7), 0)
    assert not f2.read_splats().any() and not f2.read()[..., 1:].any()
    st2 = g2.stats()
    assert st2["path_samples"] == 18 * 18 + 1  # camera samples + one photon (not traced)
