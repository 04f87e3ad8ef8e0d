"""GPU parity of textured materials and bump mapping with the oracle.

The scene of texture_scenes.py uses every texture kind of Texture.hs (Perlin
noise, fBm, cell noise with two distances, the quasi-crystal, blends, a
checker board, gradients, graph paper, RGB and grey images, scale) on every
material parameter kind, with bump maps on a uv-mapped mesh and a sphere.
The oracle and the GPU draw the same random numbers:

* depth 1 (camera ray and direct light at the first hit): the textures are
  +-*/ and floor arithmetic, bit-identical on both sides, except the
  quasi-crystal's sinf/cosf; per-pixel XYZ within 1e-3 for 97% of pixels;
* depth 5: the render tests' bar for glossy scenes (2e-3, 90%);
* the light tracer and SPPM over the same scene;
* scenes whose texture nodes break the ABI's rules are refused.
"""
import numpy as np
import pytest

from bling_gb300 import abi
from bling_gb300 import scene as S
from bling_gb300.api import BlingError
from bling_gb300.spectrum import constant, rgb_to_spectrum
from oracle.oracle import OracleScene
from texture_scenes import textured_scene

pytestmark = pytest.mark.gpu


def _render_both(gpu_ctx, sc, p, passes=1):
    g = gpu_ctx.scene(sc)
    film = gpu_ctx.film(p.width, p.height)
    o = OracleScene(sc)
    fo = None
    for k in range(passes):
        g.render_pass(film, p, k)
        fo, _ = o.render_pass(p, k, fo)
    return film.read(), fo, g.stats()


def _close(a, b, rel, frac):
    scale = np.abs(b).mean() + 1e-12
    err = np.abs(a - b) / (np.abs(b) + 1e-3 * scale)
    close = (err <= rel).all(-1)
    assert close.mean() >= frac, f"only {close.mean():.4f} of pixels within {rel}"
    ma, mb = a.mean(axis=(0, 1)), b.mean(axis=(0, 1))
    assert np.all(np.abs(ma - mb) <= 5e-3 * np.abs(mb) + 1e-9), (ma, mb)


def test_textures_at_the_first_vertex(gpu_ctx):
    sc = textured_scene(64, 44)
    p = S.render_params(64, 44, (2, 2), max_depth=1, sample_depth=2, rr_depth=2, seed=3)
    fg, fo, st = _render_both(gpu_ctx, sc, p)
    assert np.array_equal(fg[..., 0], fo[..., 0])
    _close(fg[..., 1:], fo[..., 1:], 1e-3, 0.97)
    assert st["nonfinite_drops"] == 0
    # a point light and a sky: MIS rays toward the sky are any-hit queries,
    # toward the point light none (their term is zero); same counts as the oracle
    _, st_o = OracleScene(sc).render_pass(p, 0)
    for k in ("rays_closest", "rays_any"):
        assert abs(st[k] - st_o[k]) <= 0.01 * st_o[k], (k, st[k], st_o[k])


def test_textured_paths(gpu_ctx):
    sc = textured_scene(64, 44)
    p = S.render_params(64, 44, (2, 2), max_depth=5, sample_depth=2, rr_depth=3, seed=8)
    fg, fo, st = _render_both(gpu_ctx, sc, p, passes=2)
    _close(fg[..., 1:], fo[..., 1:], 2e-3, 0.9)


def test_without_bump_maps_the_image_changes(gpu_ctx):
    p = S.render_params(48, 32, (1, 1), max_depth=1, sample_depth=2, rr_depth=2, seed=3)
    a, _, _ = _render_both(gpu_ctx, textured_scene(48, 32), p)
    b, _, _ = _render_both(gpu_ctx, textured_scene(48, 32, bump=False), p)
    assert not np.array_equal(a, b)


@pytest.mark.parametrize("max_depth", [1, 0])
def test_textured_light_pass(gpu_ctx, max_depth):
    """photons from the lights to the textured surfaces and the camera: one
    vertex (max_depth 1), and unlimited depth.  The emission directions
    (sinf/cosf) differ in the last bit, so the hit points do too; the
    textures are continuous there (the floor's checker ignores the height of
    a floor at y = 0, whose hits sit on a checker boundary)."""
    rel, frac = 2e-3, 0.9
    sc = textured_scene(48, 32)
    g = gpu_ctx.scene(sc)
    film = gpu_ctx.film(48, 32)
    g.light_pass(film, 400_000, seed=2, pass_index=0, max_depth=max_depth)
    so, st = OracleScene(sc).light_pass(48, 32, 400_000, seed=2, pass_index=0,
                                        max_depth=max_depth)
    _close(film.read_splats(), so, rel, frac)


def test_textured_sppm_pass(gpu_ctx):
    sc = textured_scene(40, 28)
    sp = abi.sppm_params(100_000, max_depth=4, radius=0.1, alpha=0.7, seed=6)
    g = gpu_ctx.scene(sc)
    film = gpu_ctx.film(40, 28)
    o = OracleScene(sc)
    f = spl = stt = None
    for k in range(2):
        g.sppm_pass(film, sp, k)
        f, spl, stt, _ = o.sppm_pass(sp, 40, 28, k, f, spl, stt)
    _close(film.read()[..., 1:], f[..., 1:], 2e-3, 0.9)
    _close(film.read_splats(), spl, 2e-3, 0.9)


def _bad(build):
    s = S.Scene()
    m = build(s)
    s.add_shape(abi.SHAPE_SPHERE, (1.0,), S.xf.identity(), m)
    s.set_perspective(S.xf.look_at((0, 0, -3), (0, 0, 0), (0, 1, 0)), 0.0, 1.0, 40.0, 8, 8)
    return s


@pytest.mark.parametrize("case", ["child_after_parent", "wrong_child_type", "slot_type",
                                  "bump_type", "too_deep", "map_kind", "no_pixels",
                                  "slot_range", "distance"])
def test_bad_texture_nodes_are_refused(gpu_ctx, case):
    def build(s):
        red = s.tex_constant(constant(0.5))
        if case == "child_after_parent":
            n = s.add_texture(S.Texture(abi.TEXN_BLEND, (red, red + 2, red + 3)))
            s.tex_constant(constant(0.2))
            s.tex_scalar(0.5)
            return s.add_material(abi.MAT_MATTE, tex={"kd": n})
        if case == "wrong_child_type":
            n = s.tex_blend(red, red, red)  # f must be scalar
            return s.add_material(abi.MAT_MATTE, tex={"kd": n})
        if case == "slot_type":
            return s.add_material(abi.MAT_MATTE, tex={"sigma": red})
        if case == "bump_type":
            return s.add_material(abi.MAT_MATTE, bump=red)
        if case == "too_deep":
            n = s.tex_scalar(1.0)
            for _ in range(abi.TEX_MAX_DEPTH):
                n = s.tex_scale(0.0, 1.0, n)
            return s.add_material(abi.MAT_MATTE, tex={"sigma": n})
        if case == "map_kind":
            n = s.add_texture(S.Texture(abi.TEXN_PERLIN, mapping=S.uv_mapping()))
            return s.add_material(abi.MAT_MATTE, tex={"sigma": n})
        if case == "no_pixels":
            n = s.add_texture(S.Texture(abi.TEXN_IMAGE, mapping=S.uv_mapping()))
            return s.add_material(abi.MAT_MATTE, tex={"kd": n})
        if case == "slot_range":
            m = s.add_material(abi.MAT_MATTE)
            s.materials[m].tex[abi.SLOT_KD] = 99
            return m
        n = s.tex_cell_noise(7)
        return s.add_material(abi.MAT_MATTE, tex={"sigma": n})
    with pytest.raises(BlingError):
        gpu_ctx.scene(_bad(build))


def test_good_texture_nodes_are_accepted(gpu_ctx):
    s = _bad(lambda s: s.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum((0.5, 0.5, 0.5)),
                                      tex={"sigma": s.tex_scale(0.1, 0.1, s.tex_perlin())}))
    gpu_ctx.scene(s)
