"""Texture expressions (Texture.hs) and bump mapping (Reflection.hs:344-377)
on the CPU: the .bling reader's texture grammar (MaterialParser.hs:120-240)
into texture nodes, known answers of the oracle's restatement, and an
oracle render of a scene that uses every kind.  The GPU parity is in
test_textures_gpu.py."""
import numpy as np
import pytest

from bling_gb300 import abi, image
from bling_gb300 import blingfile as B
from bling_gb300 import scene as S
from bling_gb300 import transform as xf
from bling_gb300.spectrum import constant, rgb_to_spectrum
from oracle.oracle import OracleScene
from texture_scenes import image_pixels, textured_scene

F = np.float32


def _one(build):
    """an oracle scene holding the nodes `build(scene)` adds; returns
    (oracle scene, the node `build` returns)"""
    s = S.Scene()
    node = build(s)
    return OracleScene(s), node


def test_perlin_is_zero_on_the_lattice_and_fbm_of_one_octave_is_perlin():
    o, (pn, fb) = _one(lambda s: (s.tex_perlin(), s.tex_fbm(1, 0.7)))
    rng = np.random.default_rng(2)
    for p in rng.integers(-300, 300, (40, 3)):
        assert o.texture(pn, p) == 0.0
    for p in rng.uniform(-5, 5, (40, 3)).astype(F):
        v = o.texture(pn, p)
        assert -1.5 < v < 1.5
        assert o.texture(fb, p) == v  # 0 + 1 * perlin
    # the permutation wraps every 256 cells (fractions exact at both places)
    p = np.array([0.25, 0.625, 0.125], F)
    assert o.texture(pn, p) == o.texture(pn, p + F(256))


def test_identity_mapping_transforms_the_point():
    o, (a, b) = _one(lambda s: (s.tex_perlin(S.identity_mapping(xf.scale(2, 2, 2))), s.tex_perlin()))
    p = np.array([0.3, 0.1, -0.4], F)
    assert o.texture(a, p) == o.texture(b, p * F(2))


def test_scale_blend_and_checker():
    def build(s):
        half = s.tex_scalar(0.25)
        sc = s.tex_scale(0.5, 2.0, half)
        r, g = s.tex_constant(rgb_to_spectrum((1, 0, 0))), s.tex_constant(rgb_to_spectrum((0, 1, 0)))
        lo, hi = s.tex_scalar(-0.1), s.tex_scalar(1.5)
        return (sc, s.tex_blend(r, g, half), s.tex_blend(r, g, lo), s.tex_blend(r, g, hi),
                s.tex_checker((1.0, 1.0, 1.0), r, g), r, g)
    o, (sc, bl, blo, bhi, chk, r, g) = _one(build)
    assert o.texture(sc, [0, 0, 0]) == F(0.5) + F(2) * F(0.25)
    R, G = rgb_to_spectrum((1, 0, 0)), rgb_to_spectrum((0, 1, 0))
    assert np.array_equal(o.texture(bl, [0, 0, 0]), R * F(0.75) + G * F(0.25))
    assert np.array_equal(o.texture(blo, [0, 0, 0]), R) and np.array_equal(o.texture(bhi, [0, 0, 0]), G)
    # floor x + floor y + floor z even: tex1 (negative sums too)
    assert np.array_equal(o.texture(chk, [0.5, 0.5, 0.5]), R)
    assert np.array_equal(o.texture(chk, [1.5, 0.5, 0.5]), G)
    assert np.array_equal(o.texture(chk, [-0.5, 0.5, 0.5]), G)
    assert np.array_equal(o.texture(chk, [-0.5, -0.5, 0.5]), R)


def test_gradient_sorts_its_steps_and_interpolates():
    A, Bc, Cc = constant(0.1), constant(0.5), constant(0.9)

    def build(s):
        f = [s.tex_scalar(x) for x in (-1.0, 0.0, 0.25, 0.5, 0.75, 1.0, 2.0)]
        return [s.tex_gradient([(1.0, Cc), (0.0, A), (0.5, Bc)], n) for n in f]
    o, nodes = _one(build)
    got = [o.texture(n, [0, 0, 0])[0] for n in nodes]
    w = (F(0.25) - F(0)) / (F(0.5) - F(0))
    assert got[0] == F(0.1) and got[1] == F(0.1) and got[5] == F(0.9) and got[6] == F(0.9)
    assert got[2] == F(0.1) * (F(1) - w) + F(0.5) * w
    assert got[3] == F(0.5)  # findIndex (> f): 0.5 is the lower end of [0.5, 1]


def test_image_texels_wrap_and_decode_like_get_pixel():
    px = image_pixels(5, 3)
    o, n = _one(lambda s: s.tex_image(px, S.uv_mapping(1, 1, 0, 0)))
    for u, v in [(0.0, 0.0), (0.21, -0.1), (0.99, -0.7), (1.25, 0.4), (-0.3, -2.2)]:
        x = int(np.floor(F(u) * F(5))) % 5
        y = int(np.floor(-F(v) * F(3))) % 3
        # unGamma: c ** 2.2 (numpy's power may differ from the C library's
        # powf in the last bit, hence the tolerance; the texel is exact)
        rgbv = tuple(np.power(F(c) / F(255), F(2.2)) for c in px[y, x])
        assert np.allclose(o.texture(n, [0, 0, 0], u, v), rgb_to_spectrum(rgbv),
                           rtol=1e-6, atol=1e-7), (u, v)


def test_grey_image_and_planar_mapping():
    px = image_pixels(4, 4, seed=9)[..., 0]
    o, n = _one(lambda s: s.tex_image_scalar(px, S.planar_mapping((1, 0, 0), (0, 0, 1), 0.5, 0)))
    p = np.array([0.3, 9.0, -0.2], F)
    u, v = p[0] + F(0.5), p[2] + F(0)
    x, y = int(np.floor(u * F(4))) % 4, int(np.floor(-v * F(4))) % 4
    assert o.texture(n, p) == F(px[y, x]) / F(255)


def test_quasi_crystal_of_one_wave():
    o, n = _one(lambda s: s.tex_crystal(1, S.uv_mapping(1, 1, 0, 0)))
    for u in np.linspace(-3, 3, 13, dtype=F):
        # (cos (1 u + 0 v) + 1) / 2; numpy's cos against the C library's cosf
        assert abs(o.texture(n, [0, 0, 0], u, 0.7) - (np.cos(u, dtype=F) + F(1)) / F(2)) <= 1e-7
    o2, n2 = _one(lambda s: s.tex_crystal(7, S.uv_mapping(5, 5, 0, 0)))
    vals = [o2.texture(n2, [0, 0, 0], u, v) for u in np.linspace(0, 1, 9) for v in np.linspace(0, 1, 9)]
    assert all(0 <= x <= 1 for x in vals)


def test_cell_noise_distance_orders():
    def build(s):
        return [s.tex_cell_noise(d) for d in (abi.DIST_EUCLIDIAN, abi.DIST_EUCLIDIAN2,
                                              abi.DIST_MANHATTAN, abi.DIST_CHEBYSHEV)]
    o, (e, e2, m, c) = _one(build)
    rng = np.random.default_rng(5)
    for p in rng.uniform(-20, 20, (60, 3)).astype(F):
        de, de2, dm, dc = (o.texture(k, p) for k in (e, e2, m, c))
        assert 0 <= dc <= de <= dm
        assert abs(de * de - de2) <= 1e-5 * max(de2, 1e-6)
        assert de < 1.8  # a cell holds at least one point


def test_reader_parses_every_texture_and_bump(tmp_path):
    px = image_pixels(4, 3)
    image.write_png(tmp_path / "wood.png", px)
    src = """
material { bumpMap bump { scale 0 0.05 tex { fbm octaves 3 omega 0.5 map { identity { scale 2 2 2 } } } }
   plastic
   kd { blend tex1 { image { file "wood.png" map { uv 2 2 0 0.5 } } }
              tex2 { gradient f { cellNoise manhattan map { identity { } } }
                     steps { 0 rgbR 0 0 0, 1 rgbR 1 1 1 } }
              f { crystal octaves 3 map { planar 1 0 0 0 0 1 0 0 } } }
   ks { checker 1 2 3 tex1 { constant rgbR 0.2 0.2 0.2 }
                      tex2 { graphPaper 0.1 map { uv 4 4 0 0 } tex1 { constant rgbR 1 1 1 }
                                                                tex2 { constant rgbR 0 0 0 } } }
   rough { scale 0.01 0.1 tex { perlin map { identity { } } } } }
prim { shape { sphere radius 1 } }
"""
    j = B.parse(src, tmp_path)
    sc = j.scene
    (m,) = sc.materials
    kinds = [t.kind for t in sc.textures]
    for k in (abi.TEXN_BLEND, abi.TEXN_IMAGE, abi.TEXN_GRADIENT, abi.TEXN_CELL_NOISE,
              abi.TEXN_CRYSTAL, abi.TEXN_CHECKER, abi.TEXN_GRAPH_PAPER, abi.TEXN_SCALE,
              abi.TEXN_PERLIN, abi.TEXN_FBM, abi.TEXN_CONSTANT):
        assert k in kinds
    for i, t in enumerate(sc.textures):  # children first
        assert all(c < i for c in t.children)
    kd = sc.textures[m.tex[abi.SLOT_KD] - 1]
    assert kd.kind == abi.TEXN_BLEND
    imgnode = sc.textures[kd.children[0]]
    assert np.array_equal(imgnode.pixels, px)
    assert imgnode.mapping == (abi.MAP_UV, (2, 2, 0, F(0.5)))
    assert sc.textures[m.tex[abi.SLOT_ROUGHNESS] - 1].kind == abi.TEXN_SCALE
    bump = sc.textures[m.bump - 1]
    assert bump.kind == abi.TEXN_SCALE and sc.textures[bump.children[0]].kind == abi.TEXN_FBM
    fbm = sc.textures[bump.children[0]]
    assert fbm.ivalue == 3 and fbm.p == (F(0.5),)
    assert np.array_equal(np.asarray(fbm.mapping[1], F), xf.scale(2, 2, 2).m)
    # the oracle renders it
    p = S.render_params(8, 8, (1, 1), max_depth=3, sample_depth=2, rr_depth=2)
    film, _ = OracleScene(sc).render_pass(p, 0)
    assert np.isfinite(film).all()


def test_textured_scene_renders_on_the_oracle_and_bump_changes_it():
    p = S.render_params(40, 28, (1, 1), max_depth=3, sample_depth=2, rr_depth=2, seed=5)
    a, st = OracleScene(textured_scene(40, 28)).render_pass(p, 0)
    b, _ = OracleScene(textured_scene(40, 28, bump=False)).render_pass(p, 0)
    assert np.isfinite(a).all() and a[..., 2].mean() > 0
    assert not np.array_equal(a, b)
