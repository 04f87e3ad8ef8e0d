"""The oracle's light tracer (Renderer/LightTracer.hs:37-110) and the camera
terms it needs, on the CPU.

* the oracle's perspective camera carries the same world-to-raster
  transform and pixel area as the host camera builder (mkProjective,
  Camera.hs:108-147), and that transform sends a camera ray's points back to
  the ray's raster position;
* a light-traced image of the Cornell room agrees with a path-traced one
  where the camera sees lit surfaces (both estimate the same radiance: the
  light tracer's splats, weighted 1 / photons, against the film's weighted
  mean), within the noise of either;
* splitting a pass's photons into ranges gives the same splat image as the
  whole pass, up to the order of float additions;
* getPixel with a splat weight (Image.hs:302-315) on the host.
"""
import ctypes as C

import numpy as np
import pytest

from bling_gb300 import abi, image
from bling_gb300 import scene as S
from bling_gb300 import transform as xf
from oracle.oracle import OracleScene, lib

F = np.float32


def _oracle_camera(look, fov, w, h):
    t = np.concatenate([look.m, look.inv]).astype(np.float32)
    out = abi.CameraDesc()
    lib().orc_camera_perspective(t.ctypes.data_as(C.POINTER(C.c_float)), 0.0, 1.0, fov, w, h,
                                 C.byref(out))
    return out


def test_oracle_camera_world_to_raster_matches_host():
    look = xf.look_at((0.5, 0.5, -1.4), (0.5, 0.5, 0.5), (0, 1, 0))
    for fov, w, h in [(40.0, 48, 48), (55.0, 64, 36), (30.0, 30, 50)]:
        c = _oracle_camera(look, fov, w, h)
        c2w, r2c, w2r, ap = xf.perspective_camera(look, 0.0, 1.0, fov, w, h, full=True)
        assert np.array_equal(np.asarray(c.w2r, F), w2r.m)
        assert F(c.pixel_area) == ap
        assert np.array_equal(np.asarray(c.r2c, F), r2c.m)


def _tp(m, p):
    m = np.asarray(m, np.float64).reshape(4, 4)
    v = m @ np.array([*p, 1.0])
    return v[:3] / v[3]


@pytest.mark.parametrize("sx,sy", [(0.5, 0.5), (10.25, 7.75), (47.0, 35.5)])
def test_world_to_raster_inverts_camera_rays(sx, sy):
    look = xf.look_at((0, 1, -4), (0, 0.5, 0), (0, 1, 0))
    c2w, r2c, w2r, ap = xf.perspective_camera(look, 0.0, 1.0, 45.0, 48, 36, full=True)
    pc = _tp(r2c.m, (sx, sy, 0))
    d = np.asarray(c2w.m, np.float64).reshape(4, 4)[:3, :3] @ (pc / np.linalg.norm(pc))
    p = _tp(c2w.m, (0, 0, 0)) + 3.7 * d
    r = _tp(w2r.m, p)
    assert abs(r[0] - sx) < 1e-4 and abs(r[1] - sy) < 1e-4
    # the pixel area of a 45 degree field over 48 x 36 pixels: (2 tan 22.5 deg * 4/3 / 48)^2
    assert np.isclose(ap, (2 * np.tan(np.radians(22.5)) * (48 / 36) / 48) ** 2, rtol=1e-5)


def test_light_tracer_agrees_with_path_tracer():
    W = H = 24
    sc = S.cornell_room(W, H)
    o = OracleScene(sc)
    p = S.cornell_params(W, H, spp_side=12, max_depth=40, rr_depth=3, seed=3)
    film, _ = o.render_pass(p, 0)
    pt = image.resolve(film)
    n = 1_500_000
    spl, st = o.light_pass(W, H, n, seed=5)
    assert st["nonfinite"] == 0 and st["splats"] > 0
    lt = image.resolve(np.zeros((H, W, 4), np.float32), spl, 1.0 / n)
    # regions of lit walls and floor (the light quad itself is seen only by
    # the path tracer: the light tracer does not connect light vertices)
    for sl in (np.s_[9:15, 9:15], np.s_[19:23, 6:18], np.s_[6:12, 6:18], np.s_[8:16, 1:4]):
        a, b = pt[sl].mean((0, 1)), lt[sl].mean((0, 1))
        assert np.all(np.abs(a - b) <= 0.05 * np.abs(a) + 1e-3), (sl, a, b)


def test_photon_ranges_sum_to_the_pass():
    W, H = 20, 16
    sc = S.cornell_room(W, H)
    o = OracleScene(sc)
    whole, st = o.light_pass(W, H, 20000, seed=9, pass_index=2, nthreads=3)
    part, st1 = o.light_pass(W, H, 20000, seed=9, pass_index=2, first=0, count=7000)
    part, st2 = o.light_pass(W, H, 20000, seed=9, pass_index=2, splats=part, first=7000)
    assert np.allclose(whole, part, rtol=1e-5, atol=1e-7)
    assert st["splats"] == st1["splats"] + st2["splats"]
    assert st["rays_closest"] == st1["rays_closest"] + st2["rays_closest"]
    # another pass index draws other photons
    other, _ = o.light_pass(W, H, 20000, seed=9, pass_index=3)
    assert not np.allclose(whole, other)


def test_max_depth_limits_the_photon_paths():
    W, H = 20, 16
    o = OracleScene(S.cornell_room(W, H))
    one, st1 = o.light_pass(W, H, 20000, seed=1, max_depth=1)
    full, st = o.light_pass(W, H, 20000, seed=1)
    # one vertex per photon: one closest-hit query each, at most one connection
    assert st1["rays_closest"] == 20000 and st1["rays_any"] <= 20000
    assert st["rays_closest"] > st1["rays_closest"]
    assert full.sum() > one.sum()


def test_resolve_with_splats():
    rng = np.random.default_rng(0)
    film = rng.random((4, 5, 4), dtype=np.float32)
    film[0, 0] = 0  # no camera samples: the splats alone
    spl = rng.random((4, 5, 3), dtype=np.float32)
    sw = F(1.0 / 3000)
    got = image.resolve(film, spl, sw)
    x = sw * spl[0, 0]
    r = F(3.240479) * x[0] - F(1.537150) * x[1] - F(0.498535) * x[2]
    assert got[0, 0, 0] == r
    w = film[1, 2, 0]
    xx = sw * spl[1, 2, 0] + film[1, 2, 1] * (F(1) / w)
    yy = sw * spl[1, 2, 1] + film[1, 2, 2] * (F(1) / w)
    zz = sw * spl[1, 2, 2] + film[1, 2, 3] * (F(1) / w)
    g = F(-0.969256) * xx + F(1.875991) * yy + F(0.041556) * zz
    assert got[1, 2, 1] == g
    assert np.array_equal(image.resolve(film), image.resolve(film, spl, 0.0))
