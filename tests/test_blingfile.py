"""The .bling reader (bling_gb300/blingfile.py) against the reference's
parser semantics (src/lib/Graphics/Bling/IO/*.hs): parser-state defaults,
newest-first primitive and light order, transforms applied to mesh vertices
with binary32 transPoint, face fans, shape constructors, materials, spectra,
renderer selection; plus an oracle render of a parsed scene.  The GPU parity
of a parsed scene is in test_render_gpu.py."""
import sys
from pathlib import Path

import numpy as np
import pytest

from bling_gb300 import abi
from bling_gb300 import blingfile as B
from bling_gb300 import transform as xf
from bling_gb300.spectrum import constant, rgb_to_spectrum
from oracle.oracle import OracleScene

F = np.float32

SCENE = """
# a small room in .bling syntax
filter mitchell 2 2 0.333333 0.333333
renderer { sampler sampled { sampler { stratified 3 2 } integrator { path maxDepth 6 sampleDepth 2 } } }
imageSize 48 32

transform { lookAt { pos 0 1 -4 look 0 0.5 0 up 0 1 0 } }
camera { perspective fov 45 lensRadius 0 focalDistance 10 }
newTransform { }

material { matte kd { constant rgbR 0.6 0.6 0.6 } sigma { constant 0 } }
prim { mesh vertexCount 4 faceCount 1
   v -2 0 -2  v 2 0 -2  v 2 0 2  v -2 0 2
   f 0 3 2 1 }

material { plastic kd { constant rgbR %20 40 c0 } ks { constant spd { 400 0.3, 700 0.5, 550 0.4 } }
           rough { constant 0.1 } }
transform { translate -0.7 0.4 0 }
prim { shape { sphere radius 0.4 } }

material { glass ior { constant 1.5 } kr { constant rgbR 1 1 1 } kt { constant rgbR 1 1 1 } }
newTransform { rotateY 30 translate 0.7 0.3 0.2 }
prim { shape { box pmin 0.3 0.3 0.3 pmax -0.3 -0.3 -0.3 } }

material { metal eta { constant rgbR 0.2 0.2 0.2 } k { constant rgbR 3.9 3.9 3.9 } rough { constant 0.05 } }
newTransform { rotateX 90 translate 0 0.01 1 }
prim { shape { disk height 0 radius 0.3 innerRadius 0.5 phiMax 400 } }

emission { rgbI 6 6 6 }
newTransform { rotateX -90 translate 0 2 0 }
prim { shape { quad 0.5 0.5 } }
emission { none }

light { directional intensity rgbI 1 0.9 0.8 normal 0.3 1 -0.4 }
light { infinite { rotateX -90 } l { constant rgbI 0.2 0.25 0.3 } }
"""


@pytest.fixture(scope="module")
def job():
    return B.parse(SCENE)


def test_parser_state_and_renderer(job):
    assert (job.width, job.height) == (48, 32)
    assert job.renderer == "path"
    assert job.sampler_kind == abi.SAMPLER_STRATIFIED and job.strata == (3, 2)
    assert (job.max_depth, job.sample_depth) == (6, 2)
    assert job.filter_kind == abi.FILTER_MITCHELL
    assert job.filter_params[0] == F(2) and job.filter_params[2] == B.f32_of_decimal("0.333333")
    p = job.params(seed=9)
    assert (p.width, p.height, p.strata_x, p.strata_y, p.max_depth, p.sample_depth, p.rr_depth,
            p.seed) == (48, 32, 3, 2, 6, 2, 7, 9)


def test_defaults_of_an_empty_file():
    j = B.parse("# nothing\n")
    assert (j.width, j.height, j.renderer, j.strata, j.max_depth, j.sample_depth) == \
        (640, 480, "path", (2, 2), 7, 3)
    assert j.filter_kind == abi.FILTER_BOX
    # defaultCamera: translate (0 0 -5), fov 90, built for 640 x 480
    c2w, r2c = xf.perspective_camera(xf.translate(0, 0, -5), 0, 1, 90, 640, 480)
    assert np.array_equal(np.asarray(j.scene.camera.c2w, F), c2w.m)
    assert np.array_equal(np.asarray(j.scene.camera.r2c, F), r2c.m)


def test_primitives_and_lights_newest_first(job):
    sc = job.scene
    # prim blocks are prepended (RenderJob.hs:52): quad, disk, box, sphere, mesh
    kinds = [sc.shapes[~v].kind if v < 0 else "mesh" for v in sc.prim_order]
    assert kinds == [abi.SHAPE_QUAD, abi.SHAPE_DISK, abi.SHAPE_BOX, abi.SHAPE_SPHERE, "mesh"]
    # lights are prepended too: infinite, then directional
    assert [l.kind for l in sc.lights] == [abi.LIGHT_INFINITE, abi.LIGHT_DIRECTIONAL]
    assert sc.lights[0].env.shape == (1, 1, 16)
    assert np.array_equal(sc.lights[0].env[0, 0], rgb_to_spectrum((F(0.2), F(0.25), F(0.3)), True))
    assert np.array_equal(sc.lights[0].w2l.m, xf.rotate_x(-90).m)
    d = sc.lights[1].vec
    assert np.array_equal(np.asarray(d, F), np.asarray(xf.normalize([F(0.3), F(1), F(-0.4)]), F))
    # only the quad emits
    em = [s.emission is not None for s in sc.shapes]
    assert em == [False, False, False, True]
    assert np.array_equal(sc.shapes[3].emission, rgb_to_spectrum((F(6), F(6), F(6)), True))


def test_mesh_vertices_and_face_fan(job):
    m = job.scene.meshes[0]
    assert m.indices.tolist() == [0, 3, 2, 0, 2, 1]  # triangulate: fan of f 0 3 2 1
    # newTransform { } before the mesh: identity, vertices unchanged
    assert m.vertices.tolist()[1] == [2.0, 0.0, -2.0]


def test_shape_transforms_and_constructors(job):
    sc = job.scene
    sphere, box, disk, quad = sc.shapes
    # "transform" composes onto the current transform: t <> current
    assert np.array_equal(sphere.o2w.m, xf.concat(xf.translate(F(-0.7), F(0.4), F(0)),
                                                  xf.identity()).m)
    # mkBox: per-axis min and max of the two corners
    assert box.params == tuple(float(F(x)) for x in [-0.3, -0.3, -0.3, 0.3, 0.3, 0.3])
    t = xf.concat(xf.rotate_y(F(30)), xf.concat(xf.translate(F(0.7), F(0.3), F(0.2)), xf.identity()))
    assert np.array_equal(box.o2w.m, t.m)
    # mkDisk: outer = max, inner = min, phiMax clamped to 360 degrees, in radians
    assert disk.params[1] == 0.5 and disk.params[2] == float(F(0.3))
    assert disk.params[3] == float(xf.radians(F(360)))
    assert quad.params == (0.5, 0.5)


def test_materials(job):
    mats = job.scene.materials
    kinds = [m.kind for m in mats]
    assert kinds == [abi.MAT_MATTE, abi.MAT_PLASTIC, abi.MAT_GLASS, abi.MAT_METAL]
    plastic = mats[1]
    assert np.array_equal(np.asarray(plastic.kd, F),
                          rgb_to_spectrum((F(0x20) / F(255), F(0x40) / F(255), F(0xc0) / F(255))))
    assert plastic.roughness == float(F(0.1))
    ks = np.asarray(plastic.ks, F)
    # pairs sorted by wavelength (400, 550, 700); band 0 ([400, 418.75]) averages
    # the samples from the first at or above 400 to the first at or above
    # 418.75 (avgSpd of an IrregularSpd); the last band takes the 700 sample
    assert ks[0] == (F(0.3) + F(0.4)) / F(2) and ks[-1] == F(0.5)
    glass = mats[2]
    assert glass.ior == 1.5 and np.array_equal(np.asarray(glass.kt, F), rgb_to_spectrum((1, 1, 1)))


def test_shiny_metal_and_translucent_matte():
    j = B.parse("material { shinyMetal kr { constant rgbR 0.9 0.8 0.5 } ks { constant rgbR 0.3 0.3 0.3 } "
                "rough { constant 0.2 } } prim { shape { sphere radius 1 } } "
                "material { transMatte kr { constant rgbR 0.4 0.4 0.4 } kt { constant rgbR 0.5 0.5 0.5 } "
                "ks { constant 0.3 } } prim { shape { sphere radius 1 } }")
    shiny, trans = j.scene.materials
    assert shiny.kind == abi.MAT_SHINY_METAL and shiny.roughness == float(F(0.2))
    assert np.array_equal(np.asarray(shiny.kd, F), rgb_to_spectrum((F(0.9), F(0.8), F(0.5))))
    assert trans.kind == abi.MAT_TRANS_MATTE and trans.sigma == float(F(0.3))
    assert np.array_equal(np.asarray(trans.kt, F), rgb_to_spectrum((F(0.5), F(0.5), F(0.5))))


def test_substrate_and_blackbody():
    j = B.parse("material { substrate kd { constant rgbR 0.5 0.4 0.3 } ks { constant rgbR 0.2 0.2 0.2 } "
                "ka { constant rgbR 0.1 0.1 0.1 } urough { constant 0.05 } vrough { constant 0.2 } "
                "depth { constant 0.5 } } prim { shape { sphere radius 1 } } "
                "material { blackbody } prim { shape { sphere radius 1 } }")
    sub, bb = j.scene.materials
    assert sub.kind == abi.MAT_SUBSTRATE and bb.kind == abi.MAT_BLACKBODY
    assert (sub.roughness, sub.sigma, sub.ior) == (float(F(0.05)), float(F(0.2)), float(F(0.5)))
    assert np.array_equal(np.asarray(sub.kt, F), rgb_to_spectrum((F(0.1), F(0.1), F(0.1))))


def test_checkerboard_and_graph_paper_diffuse_colours_are_texture_nodes():
    j = B.parse("material { matte kd { checker 2 2 2 tex1 { constant rgbR 0.8 0.8 0.8 } "
                "tex2 { constant rgbR 0.1 0.1 0.1 } } sigma { constant 0 } } "
                "prim { shape { sphere radius 1 } }")
    m = j.scene.materials[0]
    tx = j.scene.textures
    node = m.tex[abi.SLOT_KD] - 1
    assert tx[node].kind == abi.TEXN_CHECKER and tx[node].p == (2.0, 2.0, 2.0)
    a, b, _ = tx[node].children
    assert np.array_equal(tx[b].spectrum, rgb_to_spectrum((F(0.1), F(0.1), F(0.1))))
    assert tx[a].kind == tx[b].kind == abi.TEXN_CONSTANT and a < node and b < node
    j = B.parse("material { plastic kd { graphPaper 0.1 map { planar 1 0 0 0 0 1 0.5 0.25 } "
                "tex1 { constant rgbR 0.9 0.9 0.9 } tex2 { constant rgbR 0.1 0.1 0.4 } } "
                "ks { constant rgbR 0.2 0.2 0.2 } rough { constant 0.1 } }")
    g = j.scene.materials[0]
    t = j.scene.textures[g.tex[abi.SLOT_KD] - 1]
    assert t.kind == abi.TEXN_GRAPH_PAPER and t.p == (F(0.1),)
    assert t.mapping == (abi.MAP_PLANAR, (1, 0, 0, 0, 0, 1, F(0.5), F(0.25)))
    assert g.tex[abi.SLOT_KS] == 0 and g.tex[abi.SLOT_ROUGHNESS] == 0


def test_constant_spd_gives_a_flat_spectrum():
    s = B.spectrum_from_spd([(380.0, 0.25), (500.0, 0.25), (720.0, 0.25)])
    assert np.array_equal(s, constant(0.25))


def test_other_renderers_parse_and_are_named():
    j = B.parse("renderer { sppm photonCount 20000 maxDepth 10 radius 10 alpha 0.9 }")
    assert j.renderer == "sppm" and j.sppm == (20000, 10, F(10), B.f32_of_decimal("0.9"))
    sp = j.sppm_params(seed=3)
    assert (sp.photons, sp.max_depth, sp.seed) == (20000, 10, 3) and sp.alpha == F(0.9)
    assert B.parse("renderer { sppm photonCount 5 maxDepth 2 radius 1 }").sppm[3] == F(0.8)
    j = B.parse("renderer { light passPhotons 50000 }")
    assert j.renderer == "light" and j.photons_per_pass == 50000
    j = B.parse("renderer { sampler sampled { sampler { random 16 } "
                "integrator { directLighting maxDepth 3 } } }")
    assert j.renderer == "sampler/directLighting" and j.strata == (16, 1)
    assert j.sampler_kind == abi.SAMPLER_RANDOM


@pytest.mark.parametrize("src,what", [
    ("material { bumpMap bump { constant 1 } bumpMap bump { constant 1 } matte "
     "kd { constant rgbR 1 1 1 } sigma { constant 0 } }", "bumpMap"),
    ("material { matte kd { image { file \"wood.jpg\" map { uv 1 1 0 0 } } } "
     "sigma { constant 0 } }", "PNG"),
    ("prim { julia c 0 0 0 0 epsilon 0.1 iterations 4 }", "julia"),
    ("light { infinite { } l { file \"sky.png\" } }", "file"),
])
def test_unsupported_constructs_are_named(src, what):
    with pytest.raises(B.Unsupported, match=what):
        B.parse(src)


def test_syntax_errors_carry_the_line():
    with pytest.raises(B.BlingFileError, match="line 3"):
        B.parse("imageSize 8 8\n\nmaterial { plaster }\n")


def test_parsed_scene_renders_on_the_oracle(job):
    p = job.params()
    film, st = OracleScene(job.scene).render_pass(p, 0)
    assert np.isfinite(film).all()
    # the filter-padded extent (imageWindow', Image.hs:170-176): 53 x 37 pixels, 6 spp
    assert st["path_samples"] == 53 * 37 * 6
    assert film[..., 2].sum() > 0


def _examples_dir():
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    import make_example_scenes
    return make_example_scenes.source_dir()


@pytest.mark.skipif(_examples_dir() is None, reason="bling's examples directory not present")
def test_reference_cornell_box_example_parses():
    j = B.load(_examples_dir() / "cornell-box.bling")
    assert (j.width, j.height) == (480, 480)
    assert j.renderer == "sppm"  # the file's last renderer block
    assert j.scene.n_triangles == 30 and len(j.scene.shapes) == 1
    assert j.scene.shapes[0].emission is not None  # the ceiling light quad
    film, _ = OracleScene(j.scene).render_pass(
        B.Job(j.scene, 24, 24, abi.FILTER_BOX, (0, 0, 0, 0), "path", strata=(1, 1),
              max_depth=3).params(), 0)
    assert np.isfinite(film).all()


def test_wave_front_meshes(tmp_path):
    """waveFront (IO/WaveFront.hs): faces fanned, runs by usemtl, positions
    moved by the current transform, normals as read (normalised), a
    triangle's third corner taking its second corner's uv and normal, and
    the last run cut to the triangle count less its first corner index"""
    (tmp_path / "m.obj").write_text("""# two quads and a triangle
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 2 0 0
vt 0.25 0.5
vt 0.75
vn 0 0 2
vn 0 1 0
usemtl A
f 1/1/1 2/2/1 3/1/2 4/2/2
usemtl B
f 2//2 5//2 3//1
""")
    j = B.parse('newTransform { translate 0 0 5 }\n'
                'prim { waveFront "m.obj" materials { "A" { matte kd { constant rgbR 1 0 0 } '
                'sigma { constant 0 } } } }', tmp_path)
    sc = j.scene
    # runs: A from corner 0 to corner 6 (two triangles), B from corner 6 to
    # the triangle count 3 -- negative, so B's triangle is dropped
    assert sc.n_triangles == 2 and len(sc.meshes) == 1
    (m,) = sc.meshes
    assert sc.materials[m.material].kind == abi.MAT_MATTE
    assert np.array_equal(m.vertices[:3], np.array([[0, 0, 5], [1, 0, 5], [1, 1, 5]], F))
    # corners (1, 2, 3): uvs (vt1, vt2, vt2), normals (vn1, vn1, vn1)
    assert np.array_equal(m.uvs[:3], np.array([[0.25, 0.5], [0.75, 1], [0.75, 1]], F))
    assert np.array_equal(m.normals[:3], np.array([[0, 0, 1]] * 3, F))
    # the fan's second triangle: corners (1, 3, 4), uv/normal of corner 3 twice
    assert np.array_equal(m.vertices[3:], np.array([[0, 0, 5], [1, 1, 5], [0, 1, 5]], F))
    assert np.array_equal(m.normals[3:], np.array([[0, 0, 1], [0, 1, 0], [0, 1, 0]], F))
    # the material map falls back to the current material for unknown names
    j2 = B.parse('prim { waveFront "m.obj" materials { } }', tmp_path)
    assert j2.scene.materials[j2.scene.meshes[0].material].kind == abi.MAT_MATTE


def test_height_map_mesh():
    """heightMap ns nt elevation transform (Heightmap.hs:15-49)"""
    from bling_gb300 import noise
    j = B.parse("prim { heightMap 5 4 { scale 2 { fbm 0.5 octaves 2 omega 0.5 } } "
                "{ scale 3 1 3 } }")
    (m,) = j.scene.meshes
    assert len(m.vertices) == 20 and len(m.indices) == 3 * 2 * 4 * 3
    # the grid is z-major; x = i / (ns - 1), z = k / (nt - 1)
    x, z = F(2) / F(4), F(1) / F(3)
    y = F(2) * noise.fbm(2, 0.5, np.array([x], F), np.array([z], F), np.array([0.5], F))[0]
    assert np.array_equal(m.vertices[1 * 5 + 2], np.array([F(3) * x, y, F(3) * z], F))
    assert m.indices[:6].tolist() == [0, 1, 6, 0, 6, 5]
    # uvs over ns - 1 on both axes (the reference divides z by fns - 1 too)
    assert np.array_equal(m.uvs[5 * 3 + 4], np.array([F(1) / F(4), F(1) / F(4)], F))
    # shading normals: -(normalize (dx, ex + ez, dz)), so below the surface,
    # through transNormal of the scale (x and z divided by 3)
    assert (m.normals[:, 1] < 0).all()
    n0 = B._normalize_rows(np.array([[0, F(1) / F(5) + F(1) / F(4), 0]], F))
    flat = np.isclose(m.normals[:, 0], 0) & np.isclose(m.normals[:, 2], 0)
    assert np.allclose(m.normals[flat], -n0) if flat.any() else True
