"""Flat scene description and the synthetic workloads the core is measured on.

A :class:`Scene` is the host-side record a bling front end (the ``.bling``
parser, ``B/IO/RenderJob.hs``, or the DSL, ``Graphics/Bling.hs``) fills in
alongside its closure-based ``Scene``: meshes, analytic shapes with their
transforms, materials, lights and the camera, in primitive-list order.  It
lowers to the ``bling_scene_desc`` of ``include/bling_gpu.h``.

Workloads (all seeded, synthetic):

* :func:`cornell_room` -- the Cornell-style room: a unit-cube room of 5 quads
  (10 triangles), a 0.25 x 0.25 ceiling quad light of RGB radiance 15, two
  white matte boxes 0.3 and 0.6 tall rotated +-18 degrees about y, pinhole
  camera with a 40 degree field of view.
* :func:`triangle_soup` / :func:`soup_rays` -- the ray-cast microbenchmark:
  uniform-random triangles in [-1,1]^3 with edge lengths ~U(0.005, 0.05),
  rays from a sphere of radius 3 towards random points of the unit ball.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi
from . import transform as xf
from .spectrum import constant, rgb_to_spectrum

F = np.float32


@dataclass
class Mesh:
    vertices: np.ndarray          # (n, 3) float32, world space
    indices: np.ndarray           # (m,) int32, multiple of 3
    material: int
    normals: np.ndarray | None = None
    uvs: np.ndarray | None = None


@dataclass
class Shape:
    kind: int
    params: tuple
    o2w: xf.Transform
    material: int
    emission: np.ndarray | None = None


@dataclass
class Light:
    kind: int
    spectrum: np.ndarray = field(default_factory=lambda: constant(0))
    vec: tuple = (0.0, 0.0, 0.0)    # sun/sky: the sun's direction
    env: np.ndarray | None = None  # (h, w, 16) float32
    w2l: xf.Transform | None = None
    east: tuple = (0.0, 0.0, 0.0)   # sun/sky: the east direction
    turbidity: float = 0.0          # sun/sky


@dataclass
class Texture:
    """one node of a texture expression (bling_texture, Texture.hs)"""
    kind: int
    children: tuple = (-1, -1, -1)
    ivalue: int = 0
    mapping: tuple = (abi.MAP_UV, ())   # (BLING_MAP_*, numbers) of the node's mapping
    p: tuple = ()
    spectrum: np.ndarray | None = None
    steps: np.ndarray | None = None      # gradient: (n, 17) float32 (position, spectrum)
    pixels: np.ndarray | None = None     # image: (h, w, 3) or (h, w) uint8, rows top to bottom


# texture mappings (Texture.hs:147-176)
def uv_mapping(su=1.0, sv=1.0, ou=0.0, ov=0.0) -> tuple:
    """uvMapping (su, sv) (ou, ov)"""
    return (abi.MAP_UV, (su, sv, ou, ov))


def planar_mapping(vu, vv, ou=0.0, ov=0.0) -> tuple:
    """planarMapping (vu, vv) (ou, ov)"""
    return (abi.MAP_PLANAR, (*vu, *vv, ou, ov))


def identity_mapping(w2t: xf.Transform | None = None) -> tuple:
    """identityMapping3d w2t: the world-to-texture transform of the point"""
    return (abi.MAP_IDENTITY3D, tuple((w2t or xf.identity()).m.tolist()))


SLOTS = {"kd": abi.SLOT_KD, "ks": abi.SLOT_KS, "kt": abi.SLOT_KT, "eta": abi.SLOT_ETA,
         "k": abi.SLOT_K, "sigma": abi.SLOT_SIGMA, "roughness": abi.SLOT_ROUGHNESS,
         "ior": abi.SLOT_IOR}


@dataclass
class Scene:
    materials: list = field(default_factory=list)
    textures: list = field(default_factory=list)
    meshes: list = field(default_factory=list)
    shapes: list = field(default_factory=list)
    lights: list = field(default_factory=list)
    prim_order: list | None = None
    camera: abi.CameraDesc | None = None
    view: tuple | None = None  # (camera-to-world look-at transform, fov) for camera_for()

    # --- builders -------------------------------------------------------
    def add_material(self, kind, kd=None, ks=None, kt=None, eta=None, k=None, sigma=0.0,
                     roughness=0.0, ior=1.5, kd_checker=None, kd_graph=None, tex=None,
                     bump=None) -> int:
        """kd_checker: (scale (sx, sy, sz), second spectrum) makes kd the
        checkerBoard scale kd kd2 texture (Texture.hs:209-219); kd_graph:
        (lw, vu, vv, (ou, ov), line spectrum) makes it graphPaper lw
        (planarMapping (vu, vv) (ou, ov)) kd lines (Texture.hs:172-207).
        tex: {slot name: texture node} for the parameters given by texture
        expressions (slot names of SLOTS); bump: the scalar node of
        bumpMapped (Reflection.hs:344-377)."""
        m = abi.Material()
        m.kind, m.sigma, m.roughness, m.ior = kind, sigma, roughness, ior
        for name, v in (("kd", kd), ("ks", ks), ("kt", kt), ("eta", eta), ("k", k)):
            arr = constant(0) if v is None else np.asarray(v, dtype=np.float32)
            getattr(m, name)[:] = arr.tolist()
        if kd_checker is not None:
            scale, kd2 = kd_checker
            m.kd_texture = abi.TEX_CHECKER
            m.kd_tex_params[:3] = [float(np.float32(x)) for x in scale]
            m.kd2[:] = np.asarray(kd2, np.float32).tolist()
        if kd_graph is not None:
            lw, vu, vv, (ou, ov), lines = kd_graph
            m.kd_texture = abi.TEX_GRAPH_PAPER
            m.kd_tex_params[:] = [float(np.float32(x)) for x in [lw, *vu, *vv, ou, ov]]
            m.kd2[:] = np.asarray(lines, np.float32).tolist()
        for name, node in (tex or {}).items():
            m.tex[SLOTS[name]] = node + 1
        if bump is not None:
            m.bump = bump + 1
        self.materials.append(m)
        return len(self.materials) - 1

    # --- texture expressions: each returns the node's index ----------------
    def add_texture(self, t: Texture) -> int:
        self.textures.append(t)
        return len(self.textures) - 1

    def tex_constant(self, spectrum) -> int:
        return self.add_texture(Texture(abi.TEXN_CONSTANT, spectrum=np.asarray(spectrum, np.float32)))

    def tex_scalar(self, v) -> int:
        return self.add_texture(Texture(abi.TEXN_SCALAR, p=(v,)))

    def tex_blend(self, a, b, f) -> int:
        """spectrumBlend a b f"""
        return self.add_texture(Texture(abi.TEXN_BLEND, (a, b, f)))

    def tex_checker(self, scale, a, b) -> int:
        """checkerBoard (sx, sy, sz) a b"""
        return self.add_texture(Texture(abi.TEXN_CHECKER, (a, b, -1), p=tuple(scale)))

    def tex_graph_paper(self, lw, mapping, paper, lines) -> int:
        return self.add_texture(Texture(abi.TEXN_GRAPH_PAPER, (paper, lines, -1), mapping=mapping,
                                        p=(lw,)))

    def tex_gradient(self, steps, f) -> int:
        """gradient (mkGradient [(position, spectrum)]) f"""
        st = np.array([[pos, *np.asarray(sp, np.float32)] for pos, sp in steps], np.float32)
        return self.add_texture(Texture(abi.TEXN_GRADIENT, (-1, -1, f), ivalue=len(steps), steps=st))

    def tex_image(self, pixels, mapping) -> int:
        """imageTexture of an 8-bit RGB image, (h, w, 3)"""
        px = np.ascontiguousarray(pixels, np.uint8)
        assert px.ndim == 3 and px.shape[2] == 3
        return self.add_texture(Texture(abi.TEXN_IMAGE, mapping=mapping, pixels=px))

    def tex_image_scalar(self, pixels, mapping) -> int:
        """imageTexture of an 8-bit grey image, (h, w)"""
        px = np.ascontiguousarray(pixels, np.uint8)
        assert px.ndim == 2
        return self.add_texture(Texture(abi.TEXN_IMAGE_SCALAR, mapping=mapping, pixels=px))

    def tex_scale(self, a, s, t) -> int:
        """scaleTexture a s t: a + s * t"""
        return self.add_texture(Texture(abi.TEXN_SCALE, (t, -1, -1), p=(a, s)))

    def tex_perlin(self, mapping3d=None) -> int:
        return self.add_texture(Texture(abi.TEXN_PERLIN, mapping=mapping3d or identity_mapping()))

    def tex_fbm(self, octaves, omega, mapping3d=None) -> int:
        return self.add_texture(Texture(abi.TEXN_FBM, ivalue=octaves, p=(omega,),
                                        mapping=mapping3d or identity_mapping()))

    def tex_cell_noise(self, dist, mapping3d=None) -> int:
        return self.add_texture(Texture(abi.TEXN_CELL_NOISE, ivalue=dist,
                                        mapping=mapping3d or identity_mapping()))

    def tex_crystal(self, octaves, mapping) -> int:
        return self.add_texture(Texture(abi.TEXN_CRYSTAL, ivalue=octaves, mapping=mapping))

    def add_mesh(self, vertices, indices, material, normals=None, uvs=None) -> int:
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        i = np.ascontiguousarray(indices, dtype=np.int32).reshape(-1)
        n = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        uv = None if uvs is None else np.ascontiguousarray(uvs, dtype=np.float32).reshape(-1, 2)
        self.meshes.append(Mesh(v, i, material, n, uv))
        return len(self.meshes) - 1

    def add_shape(self, kind, params, o2w, material, emission=None) -> int:
        self.shapes.append(Shape(kind, tuple(params), o2w, material,
                                 None if emission is None else np.asarray(emission, np.float32)))
        return len(self.shapes) - 1

    def set_camera(self, c2w: xf.Transform, r2c: xf.Transform, lens_radius=0.0, focal_distance=1.0,
                   w2r: xf.Transform | None = None, pixel_area=0.0):
        self.camera = camera_desc(c2w, r2c, lens_radius, focal_distance, w2r, pixel_area)

    def set_perspective(self, look: xf.Transform, lens_radius, focal_distance, fov, width, height):
        """mkPerspectiveCamera look lr fd fov w h, with the world-to-raster
        transform and pixel area of sampleCam; remembered for camera_for()."""
        c2w, r2c, w2r, ap = xf.perspective_camera(look, lens_radius, focal_distance, fov, width,
                                                  height, full=True)
        self.camera = camera_desc(c2w, r2c, lens_radius, focal_distance, w2r, ap)
        self.view = (look, fov)

    def camera_for(self, width: int, height: int) -> abi.CameraDesc:
        """The scene's pinhole view built for another image size
        (mkPerspectiveCamera takes the image size, Camera.hs:108-147)."""
        look, fov = self.view
        c2w, r2c, w2r, ap = xf.perspective_camera(look, 0.0, 1.0, fov, width, height, full=True)
        return camera_desc(c2w, r2c, 0.0, 1.0, w2r, ap)

    @property
    def n_triangles(self) -> int:
        return sum(len(m.indices) // 3 for m in self.meshes)

    # --- lowering -------------------------------------------------------
    def desc(self):
        """Returns (SceneDesc, keepalive); keep the second alive while the
        descriptor is in use."""
        keep = []
        meshes = (abi.MeshDesc * max(1, len(self.meshes)))()
        for k, m in enumerate(self.meshes):
            d = meshes[k]
            d.vertices = abi.fptr(m.vertices)
            d.n_vertices = len(m.vertices)
            d.indices = abi.iptr(m.indices)
            d.n_indices = len(m.indices)
            d.normals = abi.fptr(m.normals)
            d.uvs = abi.fptr(m.uvs)
            d.material = m.material
            keep += [m.vertices, m.indices, m.normals, m.uvs]
        shapes = (abi.ShapeDesc * max(1, len(self.shapes)))()
        for k, s in enumerate(self.shapes):
            d = shapes[k]
            d.kind, d.material = s.kind, s.material
            p = list(s.params) + [0.0] * (6 - len(s.params))
            d.params[:] = p
            d.o2w[:] = s.o2w.m.tolist()
            d.w2o[:] = s.o2w.inv.tolist()
            d.emissive = 0 if s.emission is None else 1
            if s.emission is not None:
                d.emission[:] = s.emission.tolist()
        mats = (abi.Material * max(1, len(self.materials)))(*self.materials)
        lights = (abi.LightDesc * max(1, len(self.lights)))()
        for k, l in enumerate(self.lights):
            d = lights[k]
            d.kind = l.kind
            d.spectrum[:] = np.asarray(l.spectrum, np.float32).tolist()
            d.vec[:] = [float(x) for x in l.vec]
            if l.env is not None:
                env = np.ascontiguousarray(l.env, dtype=np.float32)
                keep.append(env)
                d.env = abi.fptr(env)
                d.env_h, d.env_w = env.shape[0], env.shape[1]
            w2l = l.w2l or xf.identity()
            d.w2l[:] = w2l.m.tolist()
            d.l2w[:] = w2l.inv.tolist()
            d.east[:] = [float(x) for x in l.east]
            d.turbidity = float(l.turbidity)
        order = None
        if self.prim_order is not None:
            order = np.asarray(self.prim_order, dtype=np.int32)
            keep.append(order)
        sd = abi.SceneDesc()
        sd.meshes, sd.n_meshes = meshes, len(self.meshes)
        sd.shapes, sd.n_shapes = shapes, len(self.shapes)
        sd.materials, sd.n_materials = mats, len(self.materials)
        sd.lights, sd.n_lights = lights, len(self.lights)
        sd.prim_order = abi.iptr(order)
        if self.camera is not None:
            sd.camera = self.camera
        texs = (abi.Texture * max(1, len(self.textures)))()
        for k, t in enumerate(self.textures):
            d = texs[k]
            d.kind = t.kind
            d.a, d.b, d.c = t.children
            d.ivalue = t.ivalue
            d.map_kind = t.mapping[0]
            d.map[:len(t.mapping[1])] = [float(x) for x in t.mapping[1]]
            d.p[:len(t.p)] = [float(x) for x in t.p]
            if t.spectrum is not None:
                d.spectrum[:] = np.asarray(t.spectrum, np.float32).tolist()
            if t.steps is not None:
                st = np.ascontiguousarray(t.steps, np.float32)
                keep.append(st)
                d.data = abi.fptr(st)
            if t.pixels is not None:
                px = np.ascontiguousarray(t.pixels, np.uint8)
                keep.append(px)
                d.pixels = px.ctypes.data_as(C.POINTER(C.c_uint8))
                d.height, d.width = px.shape[0], px.shape[1]
        sd.textures, sd.n_textures = texs, len(self.textures)
        keep += [meshes, shapes, mats, lights, texs]
        return sd, keep


def camera_desc(c2w: xf.Transform, r2c: xf.Transform, lens_radius=0.0, focal_distance=1.0,
                w2r: xf.Transform | None = None, pixel_area=0.0) -> abi.CameraDesc:
    c = abi.CameraDesc()
    c.c2w[:] = c2w.m.tolist()
    c.c2w_inv[:] = c2w.inv.tolist()
    c.r2c[:] = r2c.m.tolist()
    c.r2c_inv[:] = r2c.inv.tolist()
    c.lens_radius, c.focal_distance = lens_radius, focal_distance
    if w2r is not None:
        c.w2r[:] = w2r.m.tolist()
        c.pixel_area = float(pixel_area)
    return c


def crop_camera(cam: abi.CameraDesc, x0: int, y0: int) -> abi.CameraDesc:
    """The camera of a window of the image whose top-left pixel is (x0, y0):
    raster (x, y) of the window is raster (x + x0, y + y0) of the full image,
    so a film of the window's size gets exactly those pixels' camera rays."""
    r2c = xf.Transform(np.asarray(cam.r2c, np.float32), np.asarray(cam.r2c_inv, np.float32))
    r2c = xf.concat(xf.translate(x0, y0, 0), r2c)  # the shift first, then r2c
    c = abi.CameraDesc.from_buffer_copy(cam)
    c.r2c[:] = r2c.m.tolist()
    c.r2c_inv[:] = r2c.inv.tolist()
    if cam.pixel_area:
        w2r = xf.Transform(np.asarray(cam.w2r, np.float32), np.zeros(16, np.float32))
        c.w2r[:] = xf.concat(w2r, xf.translate(-x0, -y0, 0)).m.tolist()
    return c


def render_params(width, height, strata=(4, 4), max_depth=5, sample_depth=3, rr_depth=7,
                  filter_kind=abi.FILTER_BOX, filter_params=(0, 0, 0, 0), seed=1,
                  sampler=abi.SAMPLER_STRATIFIED):
    """Sampler renderer + path integrator parameters.  `strata` is (nu, nv) of
    `Stratified nu nv`; with sampler=SAMPLER_RANDOM, `mkRandomSampler spp` is
    strata=(spp, 1)."""
    p = abi.RenderParams()
    p.width, p.height = width, height
    p.sampler_kind = sampler
    p.strata_x, p.strata_y = strata
    p.max_depth, p.sample_depth, p.rr_depth = max_depth, sample_depth, rr_depth
    p.filter_kind = filter_kind
    p.filter_params[:] = [float(x) for x in filter_params]
    p.seed = seed
    return p


# ---------------------------------------------------------------- Cornell room
def _quad_tris(a, b, c, d):
    """two triangles (a, b, c), (a, c, d) of the quad a-b-c-d"""
    return [a, b, c, d], [0, 1, 2, 0, 2, 3]


def cornell_room(width=256, height=256, fov=40.0) -> Scene:
    s = Scene()
    grey = s.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum((0.75, 0.75, 0.75)))
    red = s.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum((0.63, 0.065, 0.05)))
    green = s.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum((0.14, 0.45, 0.09)))
    white = s.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum((0.75, 0.75, 0.75)))
    # room: x in [0,1] (x = 0 red, x = 1 green), y up, z in [0,1] (z = 1 back wall)
    walls_v, walls_i = [], []
    for quad in (
        [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1)],   # floor
        [(0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0)],   # ceiling
        [(0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)],   # back wall
    ):
        v, i = _quad_tris(*quad)
        walls_i += [x + len(walls_v) for x in i]
        walls_v += v
    m_grey = s.add_mesh(walls_v, walls_i, grey)
    v, i = _quad_tris((0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 1, 0))
    m_red = s.add_mesh(v, i, red)
    v, i = _quad_tris((1, 0, 0), (1, 1, 0), (1, 1, 1), (1, 0, 1))
    m_green = s.add_mesh(v, i, green)
    # ceiling light: Quad half-sizes 0.125 (area 4*sx*sy = 0.0625 = 0.25 x 0.25),
    # rotateX -90 so the light-sampled side (local -z) faces down
    light_xf = xf.rotate_x(-90) @ xf.translate(0.5, 0.999, 0.5)
    q = s.add_shape(abi.SHAPE_QUAD, (0.125, 0.125), light_xf, white,
                    emission=rgb_to_spectrum((15, 15, 15), illuminant=True))
    # boxes, rotated about y then placed on the floor
    tall = s.add_shape(abi.SHAPE_BOX, (-0.15, 0.0, -0.15, 0.15, 0.6, 0.15),
                       xf.rotate_y(18) @ xf.translate(0.33, 0.0, 0.62), white)
    short = s.add_shape(abi.SHAPE_BOX, (-0.15, 0.0, -0.15, 0.15, 0.3, 0.15),
                        xf.rotate_y(-18) @ xf.translate(0.67, 0.0, 0.33), white)
    s.prim_order = [m_grey, m_red, m_green, ~q, ~tall, ~short]
    look = xf.look_at((0.5, 0.5, -1.4), (0.5, 0.5, 0.5), (0, 1, 0))
    s.set_perspective(look, 0.0, 1.0, fov, width, height)
    return s


def cornell_params(width=256, height=256, spp_side=4, max_depth=5, rr_depth=3, seed=1):
    """16 spp (stratified 4x4), max depth 5, Russian roulette after bounce 3,
    box filter."""
    return render_params(width, height, (spp_side, spp_side), max_depth=max_depth,
                         sample_depth=3, rr_depth=rr_depth, filter_kind=abi.FILTER_BOX, seed=seed)


# ---------------------------------------------------------------- triangle soup
def _unit_vectors(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def triangle_soup(n_tris=1 << 20, seed=1, material_scene=False) -> Scene:
    """n_tris uniform-random triangles: centre ~U([-1,1]^3), two edges of
    random direction and length ~U(0.005, 0.05)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.uniform(-1, 1, size=(n_tris, 3))
    e1 = _unit_vectors(rng, n_tris) * rng.uniform(0.005, 0.05, size=(n_tris, 1))
    e2 = _unit_vectors(rng, n_tris) * rng.uniform(0.005, 0.05, size=(n_tris, 1))
    verts = np.empty((n_tris, 3, 3), dtype=np.float32)
    verts[:, 0] = c
    verts[:, 1] = c + e1
    verts[:, 2] = c + e2
    s = Scene()
    mat = s.add_material(abi.MAT_MATTE, kd=constant(0.5))
    s.add_mesh(verts.reshape(-1, 3), np.arange(3 * n_tris, dtype=np.int32), mat)
    return s


def soup_rays(n_rays=1 << 24, seed=2, any_hit=False):
    """SoA float32 (8, n): origins uniform on the sphere r=3, directions towards
    uniform points of the unit ball, tmin 0, tmax inf.  With any_hit, tmax is
    the distance to a second random point of the unit ball."""
    rng = np.random.Generator(np.random.PCG64(seed))
    o = _unit_vectors(rng, n_rays) * 3.0
    q = _unit_vectors(rng, n_rays) * rng.uniform(0, 1, size=(n_rays, 1)) ** (1 / 3)
    d = q - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.empty((8, n_rays), dtype=np.float32)
    rays[0:3] = o.T
    rays[3:6] = d.T
    rays[6] = 0.0
    rays[7] = np.inf
    if any_hit:
        q2 = _unit_vectors(rng, n_rays) * rng.uniform(0, 1, size=(n_rays, 1)) ** (1 / 3)
        rays[7] = np.linalg.norm(q2 - o, axis=1)
    return rays


# ---------------------------------------------------------------- heightfield + spheres
def _noise_lattices(seed, octaves, base_cells):
    rng = np.random.Generator(np.random.PCG64(seed))
    out, cells = [], base_cells
    for _ in range(octaves):
        out.append((cells, rng.uniform(-1, 1, size=(cells + 2, cells + 2))))
        cells *= 2
    return out


def _axis_weights(c, cells):
    """bilinear-with-smoothstep weights of 1D coordinates on a lattice axis"""
    f = np.clip(np.asarray(c, np.float64), 0, 1) * cells
    i = np.minimum(np.floor(f).astype(np.int64), cells)
    t = f - i
    s = t * t * (3 - 2 * t)
    return i, s


def value_noise(x, z, seed=7, octaves=6, amplitude=0.2, base_cells=4):
    """Seeded fractal value noise on [0,1]^2: `octaves` octaves of lattice
    values with smoothstep interpolation, frequency doubling and amplitude
    halving per octave, scaled so the sum spans +-`amplitude`.  x and z are
    broadcast point coordinates."""
    x = np.asarray(x, np.float64)
    z = np.asarray(z, np.float64)
    total = np.zeros(np.broadcast(x, z).shape)
    norm, amp = 0.0, 1.0
    for cells, lat in _noise_lattices(seed, octaves, base_cells):
        ix, sx = _axis_weights(x, cells)
        iz, sz = _axis_weights(z, cells)
        v00, v10 = lat[iz, ix], lat[iz, ix + 1]
        v01, v11 = lat[iz + 1, ix], lat[iz + 1, ix + 1]
        total += amp * ((v00 * (1 - sx) + v10 * sx) * (1 - sz) + (v01 * (1 - sx) + v11 * sx) * sz)
        norm += amp
        amp *= 0.5
    return amplitude * total / norm


def value_noise_grid(xs, zs, seed=7, octaves=6, amplitude=0.2, base_cells=4):
    """value_noise on the grid zs x xs (result [z, x]); the bilinear lattice
    interpolation factorises per axis, so each octave is two small matrix
    products."""
    total = np.zeros((len(zs), len(xs)))
    norm, amp = 0.0, 1.0
    for cells, lat in _noise_lattices(seed, octaves, base_cells):
        mats = []
        for c in (xs, zs):
            i, s = _axis_weights(c, cells)
            W = np.zeros((len(c), cells + 2))
            np.add.at(W, (np.arange(len(c)), i), 1 - s)
            np.add.at(W, (np.arange(len(c)), i + 1), s)
            mats.append(W)
        Wx, Wz = mats
        total += amp * (Wz @ lat @ Wx.T)
        norm += amp
        amp *= 0.5
    return amplitude * total / norm


def heightmap_mesh(ns, nt, elev_grid):
    """The reference's heightMap (Primitive/Heightmap.hs:15-49) in object space:
    vertices (x, elev(x, z), z) over [0,1]^2, two triangles per cell, shading
    normals -(normalize (dx, ex + ez, dz)) from central differences, and uvs
    (x/(ns-1), z/(ns-1)).  elev_grid(xs, zs) evaluates the elevation on the
    grid zs x xs."""
    fns, fnt = float(ns), float(nt)
    xs = np.arange(ns, dtype=np.float64) / (fns - 1)
    zs = np.arange(nt, dtype=np.float64) / (fnt - 1)
    X, Z = np.meshgrid(xs, zs)  # [z, x]
    Y = elev_grid(xs, zs)
    verts = np.stack([X, Y, Z], -1).reshape(-1, 3).astype(np.float32)
    ex, ez = 1 / fns, 1 / fnt
    dx = elev_grid(xs - ex, zs) - elev_grid(xs + ex, zs)
    dz = elev_grid(xs, zs - ez) - elev_grid(xs, zs + ez)
    n = np.stack([dx, np.full_like(dx, ex + ez), dz], -1)
    n = -(n / np.linalg.norm(n, axis=-1, keepdims=True))
    uvs = np.stack([X / (fns - 1), Z / (fns - 1)], -1).reshape(-1, 2).astype(np.float32)
    x = np.arange(ns - 1)
    y = np.arange(nt - 1)
    XX, YY = np.meshgrid(x, y)
    v = lambda a, b: (a + b * ns).astype(np.int64)  # noqa: E731
    tri = np.stack([v(XX, YY), v(XX + 1, YY), v(XX + 1, YY + 1),
                    v(XX, YY), v(XX + 1, YY + 1), v(XX, YY + 1)], -1)
    return verts, tri.reshape(-1).astype(np.int32), n.reshape(-1, 3).astype(np.float32), uvs


def _apply_o2w(t: xf.Transform, pts, normals=None):
    """transPoint / transNormal of a whole mesh (TriangleMesh.hs:58-59)."""
    m = t.m.reshape(4, 4).astype(np.float64)
    p = pts.astype(np.float64) @ m[:3, :3].T + m[:3, 3]
    out_n = None
    if normals is not None:
        mi = t.inv.reshape(4, 4).astype(np.float64)
        out_n = (normals.astype(np.float64) @ mi[:3, :3]).astype(np.float32)
    return p.astype(np.float32), out_n


def sky_env(width=1024, height=512, sun_dir=(0.4, 0.7, 0.3)):
    """Procedural lat-long sky (light space: +z up): zenith blue to a bright
    horizon, dark ground below, and a glow around the sun; 16-band
    illuminant spectra, (height, width, 16) float32."""
    from .spectrum import rgb_to_spectrum_array
    v = (np.arange(height) + 0.5) / height
    u = (np.arange(width) + 0.5) / width
    theta = v * np.pi
    phi = u * 2 * np.pi
    T, P = np.meshgrid(theta, phi, indexing="ij")
    d = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], -1)
    up = np.clip(d[..., 2], -1, 1)
    zen = np.array([0.25, 0.45, 1.0])
    hor = np.array([0.9, 0.9, 1.0])
    gnd = np.array([0.18, 0.16, 0.14])
    k = np.clip(up, 0, 1)[..., None] ** 0.5
    rgb = np.where(up[..., None] >= 0, hor * (1 - k) + zen * k, gnd)
    s = np.asarray(sun_dir, np.float64)
    s = np.array([s[0], s[2], s[1]]) / np.linalg.norm(s)  # world (x, y up, z) -> light (x, z, y up)
    c = np.clip((d * s).sum(-1), -1, 1)
    rgb = rgb + (np.clip(c, 0, 1) ** 64)[..., None] * np.array([6.0, 5.0, 3.5])
    return rgb_to_spectrum_array(rgb.astype(np.float32), illuminant=True)


def heightfield_scene(ns=2048, n_spheres=4096, seed=3, width=1920, height=1080, fov=45.0,
                      env_size=(1024, 512)) -> Scene:
    """ns x ns-vertex heightfield (2 (ns-1)^2 triangles) of 6-octave value noise
    (amplitude 0.2) over a 10 x 10 patch, n_spheres spheres of radius
    ~U(0.02, 0.1) scattered above it, materials per object from the seed
    (40% matte, 30% plastic with roughness ~U(0.05, 0.5), 20% metal with
    roughness ~U(0.01, 0.3), 10% glass with IOR 1.5), a procedural sky and a
    directional sun.  Metal is spectrally flat with eta = 1.2, k = 7.0
    (an aluminium-like conductor; the workload does not fix eta/k)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = Scene()
    ground = s.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum((0.35, 0.4, 0.28)))

    def elev(x, z):
        return value_noise(x, z, seed=seed)

    def elev_grid(xs, zs):
        return value_noise_grid(xs, zs, seed=seed)

    verts, idx, normals, uvs = heightmap_mesh(ns, ns, elev_grid)
    o2w = xf.scale(10, 1, 10) @ xf.translate(-5, 0, -5)
    wv, wn = _apply_o2w(o2w, verts, normals)
    m_ground = s.add_mesh(wv, idx, ground, normals=wn, uvs=uvs)
    order = [m_ground]
    kinds = rng.choice(4, size=n_spheres, p=[0.4, 0.3, 0.2, 0.1])
    px, pz = rng.uniform(-5, 5, n_spheres), rng.uniform(-5, 5, n_spheres)
    r = rng.uniform(0.02, 0.1, n_spheres)
    py = elev((px + 5) / 10, (pz + 5) / 10) + r + rng.uniform(0, 0.3, n_spheres)
    cols = rng.uniform(0.1, 0.9, (n_spheres, 3))
    for k in range(n_spheres):
        kind = int(kinds[k])
        if kind == 0:
            mat = s.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum(tuple(cols[k])))
        elif kind == 1:
            mat = s.add_material(abi.MAT_PLASTIC, kd=rgb_to_spectrum(tuple(cols[k])),
                                 ks=constant(0.5), roughness=float(rng.uniform(0.05, 0.5)))
        elif kind == 2:
            mat = s.add_material(abi.MAT_METAL, eta=constant(1.2), k=constant(7.0),
                                 roughness=float(rng.uniform(0.01, 0.3)))
        else:
            mat = s.add_material(abi.MAT_GLASS, ks=constant(1.0), kt=constant(1.0), ior=1.5)
        sh = s.add_shape(abi.SHAPE_SPHERE, (float(r[k]),),
                         xf.translate(float(px[k]), float(py[k]), float(pz[k])), mat)
        order.insert(0, ~sh)  # bling's parser prepends each prim block
    s.prim_order = order
    sun = (0.4, 0.7, 0.3)
    sd = np.asarray(sun) / np.linalg.norm(sun)
    env = sky_env(env_size[0], env_size[1], sun)
    s.lights = [S_light(abi.LIGHT_DIRECTIONAL, rgb_to_spectrum((2.6, 2.4, 2.1), illuminant=True),
                        tuple(float(v) for v in sd)),
                Light(abi.LIGHT_INFINITE, env=env, w2l=xf.rotate_x(90))]
    look = xf.look_at((0.0, 3.0, -8.0), (0.0, 0.0, 0.5), (0, 1, 0))
    s.set_perspective(look, 0.0, 1.0, fov, width, height)
    return s


def S_light(kind, spectrum, vec):
    return Light(kind, spectrum, vec=vec)


def heightfield_params(width=1920, height=1080, spp_side=8, max_depth=8, rr_depth=3, seed=1):
    return render_params(width, height, (spp_side, spp_side), max_depth=max_depth, sample_depth=3,
                         rr_depth=rr_depth, filter_kind=abi.FILTER_BOX, seed=seed)


# ---------------------------------------------------------------- batched instances
def _material_mix(s: Scene, rng, n):
    """n materials drawn like the heightfield workload's objects: 40% matte,
    30% plastic (roughness ~U(0.05, 0.5)), 20% metal (roughness
    ~U(0.01, 0.3)), 10% glass (IOR 1.5)."""
    kinds = rng.choice(4, size=n, p=[0.4, 0.3, 0.2, 0.1])
    cols = rng.uniform(0.1, 0.9, (n, 3))
    out = []
    for k in range(n):
        kind = int(kinds[k])
        if kind == 0:
            m = s.add_material(abi.MAT_MATTE, kd=rgb_to_spectrum(tuple(cols[k])))
        elif kind == 1:
            m = s.add_material(abi.MAT_PLASTIC, kd=rgb_to_spectrum(tuple(cols[k])),
                               ks=constant(0.5), roughness=float(rng.uniform(0.05, 0.5)))
        elif kind == 2:
            m = s.add_material(abi.MAT_METAL, eta=constant(1.2), k=constant(7.0),
                               roughness=float(rng.uniform(0.01, 0.3)))
        else:
            m = s.add_material(abi.MAT_GLASS, ks=constant(1.0), kt=constant(1.0), ior=1.5)
        out.append(m)
    return out


def soup_spheres_scene(n_tris, n_spheres=256, seed=1, width=256, height=256, fov=45.0,
                       env_size=(256, 128)) -> Scene:
    """A seeded random triangle soup in [-1,1]^3 plus spheres, for the batched
    workload.  Triangle edges ~U(0.5, 1.5) x 0.0275 x sqrt(2^20 / n_tris)
    (capped at 0.3), so soups of every size are about as dense as the
    1M-triangle ray-cast soup; the soup is split into 8 meshes whose
    materials, and each sphere's (radius ~U(0.02, 0.1)), follow the
    heightfield workload's mix; a procedural sky and a sun light it."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = Scene()
    scale_e = min(0.3, 0.0275 * np.sqrt((1 << 20) / max(1, n_tris)))
    c = rng.uniform(-1, 1, size=(n_tris, 3))
    e1 = _unit_vectors(rng, n_tris) * (rng.uniform(0.5, 1.5, size=(n_tris, 1)) * scale_e)
    e2 = _unit_vectors(rng, n_tris) * (rng.uniform(0.5, 1.5, size=(n_tris, 1)) * scale_e)
    verts = np.empty((n_tris, 3, 3), dtype=np.float32)
    verts[:, 0] = c
    verts[:, 1] = c + e1
    verts[:, 2] = c + e2
    n_mesh = 8
    mats = _material_mix(s, rng, n_mesh + n_spheres)
    order = []
    bounds = np.linspace(0, n_tris, n_mesh + 1).astype(np.int64)
    for k in range(n_mesh):
        part = verts[bounds[k]:bounds[k + 1]].reshape(-1, 3)
        if len(part):
            order.append(s.add_mesh(part, np.arange(len(part), dtype=np.int32), mats[k]))
    pos = rng.uniform(-1, 1, (n_spheres, 3))
    rad = rng.uniform(0.02, 0.1, n_spheres)
    for k in range(n_spheres):
        sh = s.add_shape(abi.SHAPE_SPHERE, (float(rad[k]),),
                         xf.translate(*(float(v) for v in pos[k])), mats[n_mesh + k])
        order.insert(0, ~sh)
    s.prim_order = order
    sun = (0.4, 0.7, 0.3)
    sd = np.asarray(sun) / np.linalg.norm(sun)
    s.lights = [S_light(abi.LIGHT_DIRECTIONAL, rgb_to_spectrum((2.6, 2.4, 2.1), illuminant=True),
                        tuple(float(v) for v in sd)),
                Light(abi.LIGHT_INFINITE, env=sky_env(env_size[0], env_size[1], sun),
                      w2l=xf.rotate_x(90))]
    look = xf.look_at((0.0, 0.6, -3.2), (0.0, 0.0, 0.0), (0, 1, 0))
    s.set_perspective(look, 0.0, 1.0, fov, width, height)
    return s


@dataclass
class BatchInstance:
    scene: Scene
    params: object  # abi.RenderParams
    n_tris: int


def batch_instances(n=64, seed=11, tri_range=(10_000, 2_000_000), side_range=(128, 1024),
                    strata_range=(2, 16), depth_range=(3, 10), n_spheres=256):
    """The batched workload: n scene instances, each a seeded soup plus
    spheres with a triangle count log-uniform in tri_range, a square image
    whose side is uniform in side_range, spp = sx * sy with sx, sy uniform in
    strata_range (4 ... 256 spp), and a max depth uniform in depth_range."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(n):
        nt = int(round(np.exp(rng.uniform(np.log(tri_range[0]), np.log(tri_range[1])))))
        side = int(rng.integers(side_range[0], side_range[1] + 1))
        sx = int(rng.integers(strata_range[0], strata_range[1] + 1))
        sy = int(rng.integers(strata_range[0], strata_range[1] + 1))
        depth = int(rng.integers(depth_range[0], depth_range[1] + 1))
        sc = soup_spheres_scene(nt, n_spheres=n_spheres, seed=seed * 1000 + k, width=side,
                                height=side)
        p = render_params(side, side, (sx, sy), max_depth=depth, sample_depth=3, rr_depth=3,
                          filter_kind=abi.FILTER_BOX, seed=seed * 1000 + k)
        out.append(BatchInstance(sc, p, nt))
    return out


# ---------------------------------------------------------------- white furnace
def furnace_scene(rho=0.5, width=32, height=32, le=1.0) -> Scene:
    """A Lambertian sphere of albedo rho (radius 1 at the origin) under a
    uniform environment of radiance le: light leaving the sphere is exactly
    rho * le, because every reflected ray of a convex object escapes to the
    environment; background pixels see le."""
    s = Scene()
    m = s.add_material(abi.MAT_MATTE, kd=constant(rho))
    sh = s.add_shape(abi.SHAPE_SPHERE, (1.0,), xf.identity(), m)
    s.prim_order = [~sh]
    env = np.full((8, 16, 16), le, np.float32)
    s.lights = [Light(abi.LIGHT_INFINITE, env=env, w2l=xf.identity())]
    look = xf.look_at((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), (0, 1, 0))
    s.set_perspective(look, 0.0, 1.0, 40.0, width, height)
    return s


# ---------------------------------------------------------------- serving workload
SERVING_TRIANGLES = (100_000, 200_000, 300_000, 500_000, 700_000, 1_000_000, 1_200_000, 2_000_000)


def serving_scenes(seed=31, triangles=SERVING_TRIANGLES, n_spheres=512):
    """Resident scenes of the serving workload (6M triangles in all): even
    entries a heightfield of about that many triangles plus spheres, odd
    entries a soup plus spheres, materials and lighting as in the heightfield
    workload."""
    out = []
    for k, nt in enumerate(triangles):
        if k % 2 == 0:
            ns = int(round(np.sqrt(nt / 2))) + 1
            out.append(heightfield_scene(ns=ns, n_spheres=n_spheres, seed=seed + k, width=256,
                                         height=256, env_size=(256, 128)))
        else:
            out.append(soup_spheres_scene(nt, n_spheres=n_spheres, seed=seed + k, width=256,
                                          height=256))
    return out


@dataclass
class ServingJob:
    arrival: float  # seconds after the first arrival
    scene: int
    params: object  # abi.RenderParams
    pass_index: int


def serving_jobs(n=64, rate=200.0, n_scenes=8, seed=41, side_range=(128, 1024),
                 spp_range=(16, 512), max_depth=8):
    """n jobs arriving as a Poisson process of `rate` per second, each on a
    uniformly chosen scene, with a square image whose side is log-uniform in
    side_range and spp log-uniform in spp_range (stratified sx x sy, sx the
    rounded square root)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for k in range(n):
        if k:
            t += float(rng.exponential(1.0 / rate))
        side = int(round(np.exp(rng.uniform(np.log(side_range[0]), np.log(side_range[1])))))
        spp = float(np.exp(rng.uniform(np.log(spp_range[0]), np.log(spp_range[1]))))
        sx = max(1, int(round(np.sqrt(spp))))
        sy = max(1, int(round(spp / sx)))
        p = render_params(side, side, (sx, sy), max_depth=max_depth, sample_depth=3, rr_depth=3,
                          filter_kind=abi.FILTER_BOX, seed=int(rng.integers(1, 1 << 30)))
        out.append(ServingJob(t, int(rng.integers(0, n_scenes)), p, k))
    return out
