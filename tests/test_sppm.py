"""The oracle's SPPM renderer (Renderer/SPPM.hs) on the CPU.

* an SPPM image of the Cornell room (camera samples plus photon splats with
  the reference's splat weight) agrees with a path-traced one where the
  camera sees lit surfaces, within the noise and the photon-mapping blur;
* the per-pixel radii shrink by the alpha rule where photons arrived
  (statsUpdate, SPPM.hs:272-295) and stay where none did;
* the camera pass follows specular reflection and transmission both: a
  glass sphere in front of a wall yields hit points through the glass
  only when the camera paths may bounce.
"""
import numpy as np

from bling_gb300 import abi, image
from bling_gb300 import scene as S
from bling_gb300 import transform as xf
from bling_gb300.spectrum import constant, rgb_to_spectrum
from oracle.oracle import OracleScene

F = np.float32


def _sw(photons, passes):
    sn = int(np.ceil(np.sqrt(F(photons))))
    return 1.0 / (passes * sn * sn)


def test_sppm_agrees_with_path_tracer():
    W = H = 24
    sc = S.cornell_room(W, H)
    o = OracleScene(sc)
    film, _ = o.render_pass(S.cornell_params(W, H, spp_side=12, max_depth=40, rr_depth=3, seed=3), 0)
    pt = image.resolve(film)
    sp = abi.sppm_params(200_000, max_depth=5, radius=0.02, alpha=0.7, seed=4)
    f = spl = st = None
    passes = 6
    for k in range(passes):
        f, spl, st, stats = o.sppm_pass(sp, W, H, k, f, spl, st)
        assert stats["hitpoints"] > 0 and stats["splats"] > 0 and stats["nonfinite"] == 0
    img = image.resolve(f, spl, _sw(200_000, passes))
    for sl in (np.s_[9:15, 9:15], np.s_[19:23, 6:18], np.s_[6:12, 6:18], np.s_[8:16, 1:4]):
        a, b = pt[sl].mean((0, 1)), img[sl].mean((0, 1))
        assert np.all(np.abs(a - b) <= 0.06 * np.abs(a) + 1e-3), (sl, a, b)


def test_radii_shrink_where_photons_arrive():
    W = H = 16
    o = OracleScene(S.cornell_room(W, H))
    sp = abi.sppm_params(20_000, max_depth=3, radius=0.03, alpha=0.6, seed=1)
    st0 = o.sppm_state(sp, W, H)
    r0 = st0["r2"].copy()
    assert np.all(r0 == F(0.03) * F(0.03))
    _, _, st, _ = o.sppm_pass(sp, W, H, 0, state=st0)
    shrunk = st["r2"] < r0
    assert shrunk.any() and np.all(st["r2"] <= r0)
    # N' = alpha * M after the first pass, r2' = r2 * N' / M = alpha * r2
    assert np.allclose(st["r2"][shrunk], F(0.6) * r0[shrunk], rtol=1e-6)
    assert np.all(st["n"][~shrunk] == 0) and np.all(st["m"] == 0)
    _, _, st2, _ = o.sppm_pass(sp, W, H, 1, state={k: v.copy() for k, v in st.items()})
    assert np.all(st2["r2"] <= st["r2"]) and np.all(st2["n"] >= st["n"])


def _glass_scene(w=24, h=24):
    s = S.Scene()
    wall = s.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum((0.7, 0.7, 0.7)))
    glass = s.add_material(abi.MAT_GLASS, ks=constant(1.0), kt=constant(1.0), ior=1.5)
    v = np.array([[-3, -3, 2], [3, -3, 2], [3, 3, 2], [-3, 3, 2]], np.float32)
    s.add_mesh(v, [0, 1, 2, 0, 2, 3], wall)
    sph = s.add_shape(abi.SHAPE_SPHERE, (0.8,), xf.translate(0, 0, 0), glass)
    lamp = s.add_shape(abi.SHAPE_SPHERE, (0.3,), xf.translate(0, 2, -1), wall,
                       emission=rgb_to_spectrum((6, 6, 6), illuminant=True))
    s.prim_order = [0, ~sph, ~lamp]
    s.set_perspective(xf.look_at((0, 0, -4), (0, 0, 0), (0, 1, 0)), 0.0, 1.0, 40.0, w, h)
    return s


def test_camera_pass_follows_both_specular_lobes():
    o = OracleScene(_glass_scene())
    hp = {}
    for md in (1, 6):
        sp = abi.sppm_params(1000, max_depth=md, radius=0.05, alpha=0.7)
        _, _, _, st = o.sppm_pass(sp, 24, 24, 0)
        hp[md] = st["hitpoints"]
    # depth 1: only samples whose first hit is the wall record hit points;
    # deeper trees add the wall seen through and reflected by the sphere
    assert hp[6] > hp[1] > 0
