"""A scene whose materials use every texture expression of Texture.hs and a
bump map (Reflection.hs:344-377), shared by the CPU and GPU texture tests.

Objects: a uv-mapped floor mesh, six spheres and a quad, each with its own
textured material; a point light and a constant environment."""
import numpy as np

from bling_gb300 import abi
from bling_gb300 import scene as S
from bling_gb300 import transform as xf
from bling_gb300.spectrum import constant, rgb_to_spectrum


def rgb(r, g, b):
    return rgb_to_spectrum((r, g, b))


def image_pixels(w=8, h=6, seed=4):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 256, (h, w, 3), dtype=np.uint8)


def textured_scene(w=48, h=32, bump=True):
    s = S.Scene()
    red, blue, white = s.tex_constant(rgb(0.8, 0.1, 0.1)), s.tex_constant(rgb(0.1, 0.2, 0.8)), \
        s.tex_constant(rgb(0.9, 0.9, 0.9))
    noise = s.tex_perlin(S.identity_mapping(xf.scale(4, 4, 4)))
    fbm = s.tex_fbm(4, 0.5, S.identity_mapping(xf.scale(3, 3, 3)))
    cells = s.tex_cell_noise(abi.DIST_EUCLIDIAN, S.identity_mapping(xf.scale(5, 5, 5)))
    cheb = s.tex_cell_noise(abi.DIST_CHEBYSHEV, S.identity_mapping(xf.scale(6, 6, 6)))
    crystal = s.tex_crystal(5, S.uv_mapping(12, 12, 0, 0))
    blend = s.tex_blend(red, blue, s.tex_scale(0.5, 1.0, noise))
    # the floor lies in y = 0, where floor (4 y) flips with the sign of the
    # hit point's rounding residue: the checker ignores y
    checker = s.tex_checker((4.0, 0.0, 4.0), white, blend)
    grad = s.tex_gradient([(0.0, rgb(0.1, 0.1, 0.1)), (0.3, rgb(0.9, 0.5, 0.1)),
                           (0.15, rgb(0.2, 0.7, 0.2)), (0.6, rgb(0.9, 0.9, 0.9))], cells)
    img = s.tex_image(image_pixels(), S.uv_mapping(3, 2, 0.1, 0))
    paper = s.tex_graph_paper(0.1, S.uv_mapping(8, 8, 0, 0), white, red)
    grey = s.tex_image_scalar(image_pixels(4, 4, seed=9)[..., 0], S.uv_mapping(1, 1, 0, 0))
    rough = s.tex_scale(0.02, 0.2, grey)
    wob = s.tex_scale(1.3, 0.4, crystal)
    bump_node = s.tex_scale(0.0, 0.02, fbm) if bump else None

    floor = s.add_material(abi.MAT_MATTE, tex={"kd": checker, "sigma": s.tex_scale(0.2, 0.1, noise)},
                           bump=bump_node)
    m_grad = s.add_material(abi.MAT_MATTE, tex={"kd": grad})
    m_img = s.add_material(abi.MAT_PLASTIC, ks=constant(0.3), tex={"kd": img, "roughness": rough})
    m_glass = s.add_material(abi.MAT_GLASS, ks=constant(1.0), kt=constant(1.0), tex={"ior": wob})
    m_metal = s.add_material(abi.MAT_METAL, eta=constant(1.2), k=constant(5.0),
                             tex={"roughness": s.tex_scale(0.05, 0.3, cheb)})
    m_sub = s.add_material(abi.MAT_SUBSTRATE, kd=rgb(0.3, 0.3, 0.6), ks=constant(0.1),
                           kt=constant(0.05), roughness=0.1, sigma=0.2, ior=0.3,
                           tex={"ks": paper})
    m_bumped = s.add_material(abi.MAT_PLASTIC, kd=rgb(0.6, 0.5, 0.2), ks=constant(0.4),
                              roughness=0.05, bump=s.tex_scale(0.0, 0.05, noise) if bump else None)
    m_trans = s.add_material(abi.MAT_TRANS_MATTE, tex={"kd": blend, "kt": paper, "sigma": rough})

    # a 2 x 2-quad floor with uvs over [0, 2]^2
    v = np.array([[-3, 0, -3], [0, 0, -3], [3, 0, -3], [-3, 0, 0], [0, 0, 0], [3, 0, 0],
                  [-3, 0, 3], [0, 0, 3], [3, 0, 3]], np.float32)
    uv = np.array([[0, 0], [1, 0], [2, 0], [0, 1], [1, 1], [2, 1], [0, 2], [1, 2], [2, 2]],
                  np.float32)
    idx = []
    for r in range(2):
        for c in range(2):
            a = 3 * r + c
            idx += [a, a + 1, a + 4, a, a + 4, a + 3]
    order = [s.add_mesh(v, idx, floor, uvs=uv)]
    for k, (mat, x, z) in enumerate([(m_grad, -1.6, 0.4), (m_img, -0.55, 0.4), (m_glass, 0.5, 0.2),
                                     (m_metal, 1.55, 0.4), (m_sub, -1.0, 1.5), (m_bumped, 1.0, 1.5)]):
        order.append(~s.add_shape(abi.SHAPE_SPHERE, (0.45,), xf.translate(x, 0.45, z), mat))
    order.append(~s.add_shape(abi.SHAPE_QUAD, (0.6, 0.4), xf.concat(xf.rotate_y(20), xf.translate(0, 0.6, 2.4)),
                              m_trans))
    s.prim_order = order
    s.lights = [S.Light(abi.LIGHT_POINT, rgb_to_spectrum((6, 6, 5), illuminant=True), vec=(1.0, 3.0, -1.0)),
                S.Light(abi.LIGHT_INFINITE, env=rgb_to_spectrum((0.3, 0.35, 0.4), illuminant=True)
                        .reshape(1, 1, 16), w2l=xf.rotate_x(-90))]
    s.set_perspective(xf.look_at((0.2, 2.2, -4.2), (0, 0.4, 0.6), (0, 1, 0)), 0.0, 1.0, 50.0, w, h)
    return s
