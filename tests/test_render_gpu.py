"""Parity of the GPU path integrator with the CPU oracle.

The oracle and the GPU draw the same random numbers (shared counter-based
generator), so their paths coincide until a transcendental function
(sinf/cosf/powf/acosf, not correctly rounded on either side) perturbs a
direction in the last bit.  Camera rays, first hits and direct lighting at the
first vertex are therefore bit-identical, later bounces agree to float
rounding except for the rare path that the perturbation sends to another
primitive.  The tests check:

* film weights (sample positions x filter table) are identical with the box
  filter, within 1e-5 relative otherwise (atomic summation order);
* per-pixel XYZ agree within 1e-3 relative for at least 97% of pixels
  (2e-3 / 90% for scenes with glossy and specular paths);
* image means agree within 0.5%;
* sample and ray counts agree;
* with independent random streams (different seeds), per-pixel means agree
  statistically: |z| > 4 for under 1% of pixels (z from the pass-to-pass
  variance on each side).
"""
import numpy as np
import pytest

from bling_gb300 import abi
from bling_gb300 import scene as S
from bling_gb300 import transform as xf
from bling_gb300.spectrum import constant, rgb_to_spectrum
from oracle.oracle import OracleScene, _extent

pytestmark = pytest.mark.gpu


def _render_both(gpu_ctx, sc, params, passes=1):
    g = gpu_ctx.scene(sc)
    film = gpu_ctx.film(params.width, params.height)
    o = OracleScene(sc)
    fo = None
    stats_o = []
    for k in range(passes):
        g.render_pass(film, params, k)
        fo, st = o.render_pass(params, k, fo)
        stats_o.append(st)
    return film.read(), fo, g.stats(), stats_o


def _compare(fg, fo, rel=1e-3, frac=0.97, exact_weights=False):
    # weights depend only on sample positions and the filter table; with the
    # box filter they are sums of 1.0 and equal exactly, otherwise the GPU's
    # atomic summation order changes the last bits
    if exact_weights:
        assert np.array_equal(fg[..., 0], fo[..., 0]), "film weights differ"
    else:
        assert np.allclose(fg[..., 0], fo[..., 0], rtol=1e-5, atol=1e-6), "film weights differ"
    xyz_g, xyz_o = fg[..., 1:], fo[..., 1:]
    scale = np.abs(xyz_o).mean() + 1e-12
    err = np.abs(xyz_g - xyz_o) / (np.abs(xyz_o) + 1e-3 * scale)
    close = (err <= rel).all(-1)
    assert close.mean() >= frac, f"only {close.mean():.4f} of pixels within {rel}"
    m_g, m_o = xyz_g.mean(axis=(0, 1)), xyz_o.mean(axis=(0, 1))
    assert np.all(np.abs(m_g - m_o) <= 5e-3 * np.abs(m_o) + 1e-9), (m_g, m_o)


def test_cornell_room_vs_oracle(gpu_ctx):
    sc = S.cornell_room(96, 96)
    p = S.cornell_params(96, 96, spp_side=4)
    fg, fo, st_g, st_o = _render_both(gpu_ctx, sc, p)
    _compare(fg, fo, exact_weights=True)
    assert st_g["path_samples"] == st_o[0]["path_samples"] == 98 * 98 * 16
    assert abs(st_g["rays_closest"] - st_o[0]["rays_closest"]) <= 0.01 * st_o[0]["rays_closest"]
    assert abs(st_g["rays_any"] - st_o[0]["rays_any"]) <= 0.01 * st_o[0]["rays_any"]
    assert st_g["nonfinite_drops"] == 0


def _materials_scene(w=64, h=64):
    """spheres of the four materials on a matte floor, lit by a sphere area
    light, a directional light and an environment map"""
    s = S.Scene()
    floor = s.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum((0.6, 0.6, 0.6)), sigma=0.3)
    plastic = s.add_material(abi.MAT_PLASTIC, kd=rgb_to_spectrum((0.2, 0.3, 0.7)),
                             ks=constant(0.4), roughness=0.1)
    metal = s.add_material(abi.MAT_METAL, eta=constant(0.2), k=constant(3.9), roughness=0.05)
    glass = s.add_material(abi.MAT_GLASS, ks=constant(1.0), kt=constant(1.0), ior=1.5)
    matte = s.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum((0.7, 0.3, 0.2)))
    v = np.array([[-3, 0, -3], [3, 0, -3], [3, 0, 3], [-3, 0, 3]], np.float32)
    s.add_mesh(v, [0, 1, 2, 0, 2, 3], floor)
    order = [0]
    for k, (mat, x) in enumerate([(plastic, -1.5), (metal, -0.5), (glass, 0.5), (matte, 1.5)]):
        order.append(~s.add_shape(abi.SHAPE_SPHERE, (0.45,), xf.translate(x, 0.45, 0), mat))
    order.append(~s.add_shape(abi.SHAPE_SPHERE, (0.3,), xf.translate(0, 2.5, -1), matte,
                              emission=rgb_to_spectrum((8, 8, 8), illuminant=True)))
    s.prim_order = order
    sun = S.Light(abi.LIGHT_DIRECTIONAL, rgb_to_spectrum((1.5, 1.4, 1.2), illuminant=True),
                  vec=tuple(np.array([0.3, 0.8, -0.5]) / np.linalg.norm([0.3, 0.8, -0.5])))
    env = np.zeros((16, 32, 16), np.float32)
    for y in range(16):
        env[y] = rgb_to_spectrum((0.2 + 0.02 * y, 0.3, 0.5 - 0.02 * y), illuminant=True)
    sky = S.Light(abi.LIGHT_INFINITE, env=env, w2l=xf.rotate_x(-90))
    s.lights = [sun, sky]
    c2w = xf.look_at((0, 1.5, -5), (0, 0.5, 0), (0, 1, 0))
    c2w, r2c = xf.perspective_camera(c2w, 0.0, 1.0, 40.0, w, h)
    s.set_camera(c2w, r2c)
    return s


def test_materials_and_lights_vs_oracle(gpu_ctx):
    sc = _materials_scene()
    p = S.render_params(64, 64, (3, 3), max_depth=6, sample_depth=2, rr_depth=2,
                        filter_kind=abi.FILTER_MITCHELL, filter_params=(2, 2, 1 / 3, 1 / 3))
    fg, fo, st_g, st_o = _render_both(gpu_ctx, sc, p)
    _compare(fg, fo, rel=2e-3, frac=0.9)
    assert st_g["nonfinite_drops"] == 0


@pytest.mark.parametrize("fk,fp", [(abi.FILTER_GAUSS, (1.5, 1.5, 2, 0)),
                                   (abi.FILTER_SINC, (2, 2, 3, 0)),
                                   (abi.FILTER_TRIANGLE, (1, 1, 0, 0))])
def test_filters_match(gpu_ctx, fk, fp):
    sc = S.cornell_room(40, 40)
    p = S.render_params(40, 40, (2, 2), max_depth=2, sample_depth=1, rr_depth=7,
                        filter_kind=fk, filter_params=fp)
    fg, fo, _, _ = _render_both(gpu_ctx, sc, p)
    _compare(fg, fo)


def test_heightfield_scene_vs_oracle(gpu_ctx):
    """the large-mesh workload's ingredients (heightmap mesh with shading
    normals and uvs, spheres of all four materials, sky map and sun) at a
    reduced size"""
    sc = S.heightfield_scene(ns=257, n_spheres=256, width=80, height=45, env_size=(128, 64))
    p = S.heightfield_params(80, 45, spp_side=2, max_depth=8, rr_depth=3)
    fg, fo, st_g, st_o = _render_both(gpu_ctx, sc, p)
    _compare(fg, fo, rel=2e-3, frac=0.9, exact_weights=True)
    assert st_g["nonfinite_drops"] == 0


def test_wide_bvh_layout_renders_like_the_oracle(gpu_ctx):
    """the integrator's traversal kernels over the 8-wide quantised layout"""
    from bling_gb300.api import Context
    sc = S.heightfield_scene(ns=257, n_spheres=256, width=80, height=45, env_size=(128, 64))
    p = S.heightfield_params(80, 45, spp_side=2, max_depth=8, rr_depth=3)
    wide = Context(device=0, wide_bvh=True)
    try:
        fg, fo, st_g, _ = _render_both(wide, sc, p)
    finally:
        wide.close()
    _compare(fg, fo, rel=2e-3, frac=0.9, exact_weights=True)
    assert st_g["nonfinite_drops"] == 0


def test_heightfield_full_geometry_small_image(gpu_ctx):
    """8.4M-triangle heightfield and 4096 spheres, cropped to a small image"""
    sc = S.heightfield_scene(ns=2048, n_spheres=4096, width=48, height=27, env_size=(256, 128))
    assert sc.n_triangles == 2 * 2047 * 2047
    p = S.heightfield_params(48, 27, spp_side=2, max_depth=8, rr_depth=3)
    fg, fo, st_g, st_o = _render_both(gpu_ctx, sc, p)
    _compare(fg, fo, rel=2e-3, frac=0.9, exact_weights=True)


def test_statistical_parity_independent_streams(gpu_ctx):
    sc = S.cornell_room(24, 24)
    passes = 32
    g = gpu_ctx.scene(sc)
    o = OracleScene(sc)
    film = gpu_ctx.film(24, 24)
    yg, yo = [], []
    for k in range(passes):
        pg = S.cornell_params(24, 24, spp_side=2, seed=11)
        po = S.cornell_params(24, 24, spp_side=2, seed=977)
        film.clear()
        g.render_pass(film, pg, k)
        f = film.read()
        yg.append(f[..., 2] / f[..., 0])
        fo, _ = o.render_pass(po, k)
        yo.append(fo[..., 2] / fo[..., 0])
    yg, yo = np.asarray(yg), np.asarray(yo)
    se = np.sqrt(yg.var(0, ddof=1) / passes + yo.var(0, ddof=1) / passes) + 1e-9
    z = (yg.mean(0) - yo.mean(0)) / se
    assert np.mean(np.abs(z) > 4) < 0.01, np.sort(np.abs(z).ravel())[-10:]
    assert abs(np.mean(z)) < 0.2  # no bias


@pytest.mark.parametrize("strata", [(16, 8), (32, 16)])
def test_many_strata_per_pixel_vs_oracle(gpu_ctx, strata):
    """hundreds of stratified samples per pixel and pass (the sampler's
    permutations over large strata counts).  Depth 1 (camera ray and direct
    lighting at the first vertex): with deeper paths, a last-bit difference
    of sinf/cosf sends about one path in a few hundred elsewhere, and with
    hundreds of samples per pixel most pixels hold one such path."""
    sc = S.cornell_room(24, 24)
    p = S.render_params(24, 24, strata, max_depth=1, sample_depth=3, rr_depth=3, seed=5)
    fg, fo, st_g, st_o = _render_both(gpu_ctx, sc, p, passes=2)
    _compare(fg, fo, exact_weights=True)
    assert st_g["path_samples"] == st_o[0]["path_samples"] * 2


def test_random_sampler_vs_oracle(gpu_ctx):
    """runSample (Random spp) (Sampling.hs:101-110): unstratified camera
    samples and fresh uniforms in every dimension, on both sides"""
    sc = S.cornell_room(48, 48)
    p = S.render_params(48, 48, (8, 1), max_depth=5, sample_depth=3, rr_depth=3, seed=3,
                        sampler=abi.SAMPLER_RANDOM)
    fg, fo, st_g, st_o = _render_both(gpu_ctx, sc, p)
    _compare(fg, fo, exact_weights=True)
    assert st_g["path_samples"] == st_o[0]["path_samples"] == 50 * 50 * 8


def test_parsed_bling_scene_vs_oracle(gpu_ctx):
    """a scene read from .bling text (mesh, four materials, area, directional
    and infinite lights, Mitchell filter) renders on the GPU as on the oracle"""
    from bling_gb300 import blingfile
    from test_blingfile import SCENE
    job = blingfile.parse(SCENE)
    fg, fo, st_g, st_o = _render_both(gpu_ctx, job.scene, job.params(seed=4))
    _compare(fg, fo, rel=2e-3, frac=0.9)
    assert st_g["path_samples"] == st_o[0]["path_samples"]
    assert st_g["nonfinite_drops"] == 0
    # MIS rays: closest-hit queries toward the area light, any-hit toward the
    # sky, none toward the directional light; the oracle counts alike
    for k in ("rays_closest", "rays_any"):
        assert abs(st_g[k] - st_o[0][k]) <= 0.01 * st_o[0][k], (k, st_g[k], st_o[0][k])


def test_mirror_material_vs_oracle(gpu_ctx):
    """mirrorMaterial (specRefl frNoOp kr, Material.hs:68-72): a mirror sphere
    and a mirror quad over a matte floor under a sky and a sun"""
    sc = _materials_scene()
    mirror = sc.add_material(abi.MAT_MIRROR, ks=rgb_to_spectrum((0.9, 0.8, 0.7)))
    sc.shapes[1].material = mirror  # the metal sphere becomes a mirror
    q = sc.add_shape(abi.SHAPE_QUAD, (0.6, 0.4), xf.rotate_y(20) @ xf.translate(0.0, 0.5, 1.2),
                     mirror)
    sc.prim_order = sc.prim_order + [~q]
    p = S.render_params(64, 64, (3, 3), max_depth=6, sample_depth=2, rr_depth=2, seed=7)
    fg, fo, st_g, st_o = _render_both(gpu_ctx, sc, p)
    _compare(fg, fo, rel=2e-3, frac=0.9, exact_weights=True)
    assert st_g["nonfinite_drops"] == 0


def test_shiny_metal_and_translucent_matte_vs_oracle(gpu_ctx):
    """mkShinyMetal (conductor Fresnel approximated from the colours) and
    translucentMatte (a diffuse BRDF and the same lobe as a BTDF, light seen
    through a thin translucent quad)"""
    sc = _materials_scene()
    shiny = sc.add_material(abi.MAT_SHINY_METAL, kd=rgb_to_spectrum((0.95, 0.8, 0.4)),
                            ks=rgb_to_spectrum((0.5, 0.45, 0.3)), roughness=0.1)
    trans = sc.add_material(abi.MAT_TRANS_MATTE, kd=rgb_to_spectrum((0.3, 0.4, 0.3)),
                            kt=rgb_to_spectrum((0.7, 0.6, 0.5)), sigma=0.2)
    trans_l = sc.add_material(abi.MAT_TRANS_MATTE, kd=rgb_to_spectrum((0.5, 0.5, 0.5)),
                              kt=rgb_to_spectrum((0.9, 0.9, 0.9)))
    sc.shapes[1].material = shiny   # the metal sphere
    sc.shapes[0].material = trans   # the plastic sphere
    q = sc.add_shape(abi.SHAPE_QUAD, (0.8, 0.8), xf.rotate_x(-90) @ xf.translate(0.0, 1.6, -1.0),
                     trans_l)  # a translucent ceiling panel under the sphere light
    sc.prim_order = sc.prim_order + [~q]
    p = S.render_params(64, 64, (3, 3), max_depth=6, sample_depth=2, rr_depth=2, seed=13)
    fg, fo, st_g, st_o = _render_both(gpu_ctx, sc, p)
    _compare(fg, fo, rel=2e-3, frac=0.9, exact_weights=True)
    assert st_g["nonfinite_drops"] == 0


def test_lights_and_thin_lens_vs_oracle(gpu_ctx):
    """a point light, disk, cylinder and box area lights (shape sampling of
    each kind, Shape.hs:333-409), and a thin-lens camera (lens samples,
    concentricSampleDisk, Camera.hs:49-68)"""
    s = S.Scene()
    grey = s.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum((0.6, 0.6, 0.6)))
    plastic = s.add_material(abi.MAT_PLASTIC, kd=rgb_to_spectrum((0.3, 0.5, 0.2)),
                             ks=constant(0.3), roughness=0.2)
    v = np.array([[-4, 0, -4], [4, 0, -4], [4, 0, 4], [-4, 0, 4]], np.float32)
    s.add_mesh(v, [0, 1, 2, 0, 2, 3], grey)
    order = [0]
    order.append(~s.add_shape(abi.SHAPE_SPHERE, (0.5,), xf.translate(0.6, 0.5, 0.4), plastic))
    em = rgb_to_spectrum((4, 3.5, 3), illuminant=True)
    order.append(~s.add_shape(abi.SHAPE_DISK, (0.0, 0.4, 0.1, 2 * np.pi),
                              xf.rotate_x(90) @ xf.translate(-1.0, 2.0, 0.0), grey, emission=em))
    order.append(~s.add_shape(abi.SHAPE_CYLINDER, (0.08, -0.5, 0.5, 2 * np.pi),
                              xf.rotate_x(90) @ xf.translate(1.5, 0.6, -0.5), grey, emission=em))
    order.append(~s.add_shape(abi.SHAPE_BOX, (-0.1, -0.1, -0.1, 0.1, 0.1, 0.1),
                              xf.translate(-0.6, 0.15, -0.6), grey, emission=em))
    s.prim_order = order
    s.lights = [S.Light(abi.LIGHT_POINT, rgb_to_spectrum((2, 2, 2), illuminant=True),
                        vec=(0.0, 2.5, -1.0))]
    look = xf.look_at((0, 1.6, -4), (0, 0.4, 0), (0, 1, 0))
    c2w, r2c = xf.perspective_camera(look, 0.08, 4.0, 45.0, 64, 48)
    s.set_camera(c2w, r2c, lens_radius=0.08, focal_distance=4.0)
    p = S.render_params(64, 48, (3, 3), max_depth=5, sample_depth=3, rr_depth=3, seed=11)
    fg, fo, st_g, st_o = _render_both(gpu_ctx, s, p)
    _compare(fg, fo, rel=2e-3, frac=0.9, exact_weights=True)
    assert st_g["nonfinite_drops"] == 0
    assert fg[..., 2].sum() > 0


def test_film_resolve_and_png(gpu_ctx, tmp_path):
    """bling_film_resolve (getPixel + xyzToRgb on the read film) equals the
    host restatement, and the 8-bit image round-trips through a PNG"""
    from bling_gb300 import image
    sc = S.cornell_room(40, 30)
    g = gpu_ctx.scene(sc)
    film = gpu_ctx.film(40, 30)
    g.render_pass(film, S.cornell_params(40, 30, spp_side=2), 0)
    rgb = film.resolve()
    assert np.array_equal(rgb, image.resolve(film.read()))
    img = image.to_rgb8(rgb)
    image.write_png(tmp_path / "cornell.png", img)
    assert np.array_equal(image.read_png(tmp_path / "cornell.png"), img)
    assert img.mean() > 10


def test_passes_accumulate(gpu_ctx):
    sc = S.cornell_room(32, 32)
    p = S.cornell_params(32, 32, spp_side=2)
    fg, fo, st_g, _ = _render_both(gpu_ctx, sc, p, passes=3)
    _compare(fg, fo, exact_weights=True)
    assert st_g["path_samples"] == 3 * 34 * 34 * 4


def test_substrate_and_blackbody_vs_oracle(gpu_ctx):
    """mkSubstrate (FresnelBlend with the anisotropic microfacet distribution,
    with and without a coating depth) and blackBodyMaterial (no BxDFs: paths
    end there)"""
    sc = _materials_scene()
    sub = sc.add_material(abi.MAT_SUBSTRATE, kd=rgb_to_spectrum((0.6, 0.3, 0.2)), ks=constant(0.15),
                          kt=constant(0.0), roughness=0.05, sigma=0.05, ior=0.0)
    aniso = sc.add_material(abi.MAT_SUBSTRATE, kd=rgb_to_spectrum((0.2, 0.4, 0.6)),
                            ks=constant(0.3), kt=rgb_to_spectrum((0.3, 0.1, 0.1)), roughness=0.02,
                            sigma=0.4, ior=0.3)
    black = sc.add_material(abi.MAT_BLACKBODY)
    sc.shapes[0].material = sub     # the plastic sphere
    sc.shapes[1].material = aniso   # the metal sphere
    sc.shapes[3].material = black   # the matte sphere
    p = S.render_params(64, 64, (3, 3), max_depth=6, sample_depth=2, rr_depth=2, seed=17)
    fg, fo, st_g, st_o = _render_both(gpu_ctx, sc, p)
    _compare(fg, fo, rel=2e-3, frac=0.9, exact_weights=True)
    assert st_g["nonfinite_drops"] == 0


def test_checkerboard_diffuse_colour_vs_oracle(gpu_ctx):
    """checkerBoard kd textures (Texture.hs:209-219) on a matte floor, a
    plastic sphere and a substrate sphere: the colour follows the parity of
    floor(x sx) + floor(y sy) + floor(z sz) at the shading point"""
    sc = _materials_scene()
    floor = sc.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum((0.8, 0.8, 0.8)), sigma=0.3,
                            kd_checker=((2.0, 2.0, 2.0), rgb_to_spectrum((0.1, 0.2, 0.1))))
    plastic = sc.add_material(abi.MAT_PLASTIC, kd=rgb_to_spectrum((0.7, 0.2, 0.2)), ks=constant(0.3),
                              roughness=0.1,
                              kd_checker=((8.0, 8.0, 8.0), rgb_to_spectrum((0.2, 0.2, 0.7))))
    sub = sc.add_material(abi.MAT_SUBSTRATE, kd=rgb_to_spectrum((0.6, 0.5, 0.2)), ks=constant(0.1),
                          kt=constant(0.0), roughness=0.1, sigma=0.1, ior=0.0,
                          kd_checker=((5.0, 0.0, 5.0), rgb_to_spectrum((0.1, 0.1, 0.1))))
    sc.meshes[0].material = floor
    sc.shapes[0].material = plastic
    sc.shapes[3].material = sub
    p = S.render_params(64, 64, (3, 3), max_depth=5, sample_depth=2, rr_depth=2, seed=23)
    fg, fo, st_g, st_o = _render_both(gpu_ctx, sc, p)
    _compare(fg, fo, rel=2e-3, frac=0.9, exact_weights=True)


def test_textured_kd_of_other_materials_is_refused(gpu_ctx):
    s = S.Scene()
    m = s.add_material(abi.MAT_METAL, eta=constant(0.2), k=constant(3.9), roughness=0.1,
                       kd_checker=((1.0, 1.0, 1.0), constant(0.5)))
    s.add_shape(abi.SHAPE_SPHERE, (1.0,), xf.identity(), m)
    with pytest.raises(Exception):
        gpu_ctx.scene(s)


def test_graph_paper_diffuse_colour_vs_oracle(gpu_ctx):
    """graphPaper with a planar mapping (Texture.hs:172-207) on the matte
    floor and a plastic sphere"""
    sc = _materials_scene()
    floor = sc.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum((0.9, 0.9, 0.85)),
                            kd_graph=(0.08, (2.0, 0.0, 0.0), (0.0, 0.0, 2.0), (0.25, 0.5),
                                      rgb_to_spectrum((0.1, 0.1, 0.5))))
    plastic = sc.add_material(abi.MAT_PLASTIC, kd=rgb_to_spectrum((0.7, 0.6, 0.2)), ks=constant(0.3),
                              roughness=0.1,
                              kd_graph=(0.2, (0.0, 6.0, 0.0), (6.0, 0.0, 0.0), (0.0, 0.0),
                                        rgb_to_spectrum((0.1, 0.1, 0.1))))
    sc.meshes[0].material = floor
    sc.shapes[0].material = plastic
    p = S.render_params(64, 64, (3, 3), max_depth=5, sample_depth=2, rr_depth=2, seed=29)
    fg, fo, st_g, st_o = _render_both(gpu_ctx, sc, p)
    _compare(fg, fo, rel=2e-3, frac=0.9, exact_weights=True)


def test_first_dropped_sample_is_reported(gpu_ctx):
    """a point light whose band 3 is NaN makes every lit sample's radiance
    NaN, which the film drops (Image.hs:253-256); the scene statistics name
    the pass and its lowest dropped sample (pixels row by row, then sample
    number), which is the first non-finite sample of the oracle's replay"""
    s = S.Scene()
    m = s.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum((0.5, 0.5, 0.5)))
    s.add_mesh(np.array([[-4, 0, -4], [4, 0, -4], [4, 0, 4], [-4, 0, 4]], np.float32),
               [0, 1, 2, 0, 2, 3], m)
    bad = constant(2.0)
    bad[3] = np.nan
    s.lights = [S.Light(abi.LIGHT_POINT, bad, vec=(0.0, 2.0, 0.0))]
    w, h = 24, 16
    s.set_perspective(xf.look_at((0, 1, -6), (0, 0.9, 0), (0, 1, 0)), 0.0, 1.0, 50.0, w, h)
    p = S.render_params(w, h, (2, 2), max_depth=2, sample_depth=3, rr_depth=3, seed=3)
    g = gpu_ctx.scene(s)
    assert g.stats()["nonfinite_pass"] == -1
    film = gpu_ctx.film(w, h)
    g.render_pass(film, p, 7)
    st = g.stats()
    o = OracleScene(s)
    first, dropped = None, 0
    x0, x1, y0, y1 = _extent(p)  # the sample extent: a pixel wider than the image
    for y in range(y0, y1 + 1):
        for x in range(x0, x1 + 1):
            for n in range(4):
                spec = o.sample_li(p, 7, x, y, n)[2]
                if not np.isfinite(spec).all():
                    dropped += 1
                    first = first or (x, y, n)
    assert first is not None and first[1] > y0  # the top rows see only the empty sky
    assert st["nonfinite_drops"] == dropped
    assert st["nonfinite_pass"] == 7
    assert (*st["nonfinite_pixel"], st["nonfinite_sample"]) == first


def test_sunsky_light_vs_oracle(gpu_ctx):
    """the sun/sky map (SunSky.hs) evaluated on the device wherever the
    light's le and sample need it; the importance distribution over its
    640 x 480 raster"""
    from test_sunsky import sunsky_scene
    sc = sunsky_scene(64, 48)
    p = S.render_params(64, 48, (2, 2), max_depth=5, sample_depth=2, rr_depth=2, seed=11)
    fg, fo, st_g, st_o = _render_both(gpu_ctx, sc, p)
    _compare(fg, fo, rel=2e-3, frac=0.9, exact_weights=True)
    assert st_g["nonfinite_drops"] == 0
    assert fo[..., 2].mean() > 0


@pytest.mark.parametrize("scene", ["cornell", "heightfield"])
def test_ray_binning_renders_the_same(gpu_ctx, scene):
    """BLING_FLAG_BIN_RAYS only reorders which warp traces which ray: the
    film is the same up to the order of its float additions, and the ray and
    sample counts are equal."""
    from bling_gb300.api import Context
    if scene == "cornell":
        sc, p = S.cornell_room(64, 64), S.cornell_params(64, 64, spp_side=4)
    else:
        sc = S.heightfield_scene(ns=257, n_spheres=64, width=64, height=36, env_size=(64, 32))
        p = S.heightfield_params(64, 36, spp_side=4, max_depth=8)
    ctx = Context(device=0, bin_rays=True)
    try:
        ga, gb = gpu_ctx.scene(sc), ctx.scene(sc)
        fa, fb = gpu_ctx.film(p.width, p.height), ctx.film(p.width, p.height)
        ga.render_pass(fa, p, 0)
        gb.render_pass(fb, p, 0)
        a, b = fa.read(), fb.read()
        assert np.array_equal(a[..., 0], b[..., 0])
        scale = float(np.abs(a[..., 1:]).max()) + 1e-30
        assert np.allclose(a[..., 1:], b[..., 1:], rtol=1e-5, atol=1e-6 * scale)
        sa, sb = ga.stats(), gb.stats()
        for k in ("rays_closest", "rays_any", "path_samples", "nonfinite_drops"):
            assert sa[k] == sb[k], k
    finally:
        ctx.close()
