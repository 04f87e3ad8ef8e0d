"""Reader for bling's ``.bling`` scene files: the flat scene record a bling
front end hands to the GPU path integrator.

Mirrors the reference's parser (``src/lib/Graphics/Bling/IO/*.hs``): the same
objects, blocks and keywords, the same parser state and its defaults
(``RenderJob.hs:24-33``), and the same order of primitives and lights, so a
file renders through :class:`~bling_gb300.api.GpuPathRenderer` with the
primitive IDs and light list ``mkScene`` would build (``Scene.hs:37-43``).
Numbers are rounded to binary32 once, as GHC's ``read :: Float`` does, and
transforms, spectra and meshes are built with the binary32 restatements of
``Transform.hs`` and ``Spectrum.hs`` (``transform.py``, ``spectrum.py``).

The subset is what the GPU path renders:

* objects: ``filter``, ``imageSize``, ``renderer``, ``transform``,
  ``newTransform``, ``camera``, ``light``, ``material``, ``emission``,
  ``prim``;
* primitives: ``mesh``, ``shape`` (box, cylinder, disk, quad, sphere),
  ``heightMap`` (fbm and scale elevation maps, tessellated on the host) and
  ``waveFront`` (Wavefront .obj files with a material map);
* materials: matte, plastic, metal, glass, mirror, shinyMetal, transMatte,
  substrate, blackbody and bumpMap, every parameter a texture: constant,
  blend, checker, gradient, graphPaper and (PNG) image spectra; constant,
  scale, perlin, fbm, cellNoise, crystal and (PNG) image scalars; uv, planar
  and identity mappings;
* lights: directional, point, and infinite with a ``constant`` or ``sunSky``
  map;
* spectra: ``rgbR``/``rgbI`` (decimal or ``%rrggbb``), ``spd { l v, ... }``,
  ``temp``, ``blackbody``;
* the renderers ``sampler`` (``stratified``/``random`` with the ``path``
  integrator), ``light`` and ``sppm``.

Anything else raises :class:`Unsupported` naming the construct; a file whose
renderer is not the path integrator parses, and :attr:`Job.renderer` names
the renderer it asked for.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import abi, image, noise
from . import transform as xf
from .gen_spectrum_tables import BANDS, LAMBDA_END, LAMBDA_START, f32_of_decimal, lerp
from .scene import Light, Scene, identity_mapping, planar_mapping, render_params, uv_mapping
from .spectrum import constant, rgb_to_spectrum

F = np.float32


class BlingFileError(ValueError):
    """A syntax error in a .bling file."""


@dataclass(frozen=True)
class _Node:
    """a parsed texture that is not constant: its node in Scene.textures"""
    index: int


class Unsupported(BlingFileError):
    """A construct the reference parses but the GPU path does not render."""


@dataclass
class Job:
    """A parsed render job: the scene, the image size and the renderer."""
    scene: Scene
    width: int
    height: int
    filter_kind: int
    filter_params: tuple
    renderer: str                      # "path", or the reference renderer the file selects
    sampler_kind: int = abi.SAMPLER_STRATIFIED
    strata: tuple = (2, 2)             # (nu, nv), or (spp, 1) for the random sampler
    max_depth: int = 7                 # mkPathIntegrator 7 3 (IntegratorParser.hs)
    sample_depth: int = 3
    photons_per_pass: int = 0          # renderer { light passPhotons N } (RendererParser.hs:28-30)
    sppm: tuple | None = None          # (photonCount, maxDepth, radius, alpha) (RendererParser.hs:40-45)
    camera_view: tuple | None = None   # (camera-to-world, lens radius, focal distance, fov)

    def camera_for(self, width: int, height: int) -> abi.CameraDesc:
        """the file's camera built for another image size (mkPerspectiveCamera
        takes the image size, Camera.hs:108-147), e.g. for a reduced render"""
        from .scene import camera_desc
        c2w, lr, fd, fov = self.camera_view
        c2w_, r2c, w2r, ap = xf.perspective_camera(c2w, lr, fd, fov, width, height, full=True)
        return camera_desc(c2w_, r2c, lr, fd, w2r, ap)

    def sppm_params(self, seed: int = 1) -> abi.SppmParams:
        """bling_sppm_params of a `renderer { sppm ... }` job (mkSPPM n md r alpha)"""
        n, md, r, a = self.sppm
        return abi.sppm_params(n, md, r, a, filter_kind=self.filter_kind,
                               filter_params=self.filter_params, seed=seed)

    def params(self, seed: int = 1, rr_depth: int = 7) -> abi.RenderParams:
        """bling_render_params of the job's sampler renderer and path
        integrator (Russian roulette after depth 7 as in Path.hs:68)."""
        return render_params(self.width, self.height, self.strata, max_depth=self.max_depth,
                             sample_depth=self.sample_depth, rr_depth=rr_depth,
                             filter_kind=self.filter_kind, filter_params=self.filter_params,
                             seed=seed, sampler=self.sampler_kind)


# ---------------------------------------------------------------- tokens
# ws = spaces and '#' comments (ParserCore.hs:111-119); words are alphaNum
# runs (pString); numbers are [+-]digits[.digits] (flt')
_TOKEN = re.compile(r"""
    (?P<ws>\s+|\#[^\n]*)
  | (?P<str>"(?:[^"\\\r\n]|\\[^\r\n])*")
  | (?P<hex>%[0-9A-Fa-f]{2}(?:\s*[0-9A-Fa-f]{2}){2})
  | (?P<num>[+-]?\d+(?:\.\d*)?(?![A-Za-z]))
  | (?P<word>[A-Za-z0-9]+)
  | (?P<sym>[{},])
""", re.X)


class _Tokens:
    def __init__(self, text: str):
        self.toks = []
        pos = 0
        line = 1
        while pos < len(text):
            m = _TOKEN.match(text, pos)
            if not m:
                raise BlingFileError(f"line {line}: unexpected character {text[pos]!r}")
            kind = m.lastgroup
            if kind != "ws":
                self.toks.append((kind, m.group(kind), line))
            line += m.group(0).count("\n")
            pos = m.end()
        self.i = 0

    def peek(self):
        return self.toks[self.i] if self.i < len(self.toks) else (None, None, -1)

    def next(self):
        t = self.peek()
        if t[0] is None:
            raise BlingFileError("unexpected end of file")
        self.i += 1
        return t

    def error(self, msg):
        return BlingFileError(f"line {self.peek()[2]}: {msg}")

    def word(self) -> str:
        kind, val, line = self.next()
        if kind not in ("word", "num"):
            raise BlingFileError(f"line {line}: expected a name, got {val!r}")
        return val

    def expect(self, what: str):
        kind, val, line = self.next()
        if val != what:
            raise BlingFileError(f"line {line}: expected {what!r}, got {val!r}")

    def flt(self) -> np.float32:
        kind, val, line = self.next()
        if kind != "num":
            raise BlingFileError(f"line {line}: expected a number, got {val!r}")
        return f32_of_decimal(val if "." not in val or not val.endswith(".") else val + "0")

    def integ(self) -> int:
        kind, val, line = self.next()
        if kind != "num" or not val.isdigit():
            raise BlingFileError(f"line {line}: expected a non-negative integer, got {val!r}")
        return int(val)

    def vec(self):
        return [self.flt(), self.flt(), self.flt()]

    def named_flt(self, name):
        self.expect(name)
        return self.flt()

    def named_int(self, name):
        self.expect(name)
        return self.integ()

    def named_vec(self, name):
        self.expect(name)
        return self.vec()

    def at(self, val) -> bool:
        return self.peek()[1] == val

    def block(self, body):
        """pBlock: '{' body '}'"""
        self.expect("{")
        r = body()
        self.expect("}")
        return r

    def named_block(self, name, body):
        self.expect(name)
        return self.block(body)


# ---------------------------------------------------------------- binary32 helpers
def _ghc_min(a, b):
    return a if a <= b else b


def _ghc_max(a, b):
    return b if a <= b else a


def _clamp(v, lo, hi):
    """clamp (Math.hs:78-87)"""
    return lo if v < lo else (hi if v > hi else v)


def trans_point(t: xf.Transform, p):
    """transPoint (Transform.hs:246-256): left-to-right binary32 sums; the
    homogeneous divide only when w != 1."""
    m = t.m
    x, y, z = F(p[0]), F(p[1]), F(p[2])

    def row(r):
        return ((m[4 * r] * x + m[4 * r + 1] * y) + m[4 * r + 2] * z) + m[4 * r + 3]
    xp, yp, zp, wp = row(0), row(1), row(2), row(3)
    if wp == F(1):
        return [xp, yp, zp]
    return [xp / wp, yp / wp, zp / wp]


def _avg_irregular_spd(ls, vs, l0, l1):
    """avgSpd (IrregularSpd ls vs) l0 l1 (Spectrum.hs:307-314)"""
    if l1 <= ls[0]:
        return vs[0]
    if l0 >= ls[-1]:
        return vs[-1]

    def find(lim, default):
        for k, l in enumerate(ls):
            if l >= lim:
                return k
        return default
    i0 = find(l0, 0)
    i1 = find(l1, len(vs) - 1)
    sl = vs[i0:i1 + 1]
    acc = F(0)
    for v in sl:
        acc = acc + v
    return acc / F(len(sl))


def spectrum_from_spd(pairs) -> np.ndarray:
    """fromSpd (mkSpd pairs) (Spectrum.hs:199-208, 329-335): the pairs sorted
    by wavelength (a stable sort, as sortBy), each band the plain average of
    the samples from the first at or above its lower edge to the first at or
    above its upper edge."""
    if not pairs:
        raise BlingFileError("empty SPD")
    srt = sorted(pairs, key=lambda p: p[0])
    ls = [F(l) for l, _ in srt]
    vs = [F(v) for _, v in srt]
    out = []
    for i in range(BANDS):
        l0 = lerp(F(i) / F(BANDS), LAMBDA_START, LAMBDA_END)
        l1 = lerp(F(i + 1) / F(BANDS), LAMBDA_START, LAMBDA_END)
        out.append(_avg_irregular_spd(ls, vs, l0, l1))
    return np.asarray(out, np.float32)


def _planck(temp, w):
    """planck (Spectrum.hs:491-493) in binary32; w'^^(-5) = recip of GHC's
    (^) by squaring, ((w'*w')*(w'*w'))*w'."""
    w1 = F(w) * F(1e-9)
    w2 = w1 * w1
    p5 = (w2 * w2) * w1
    num = F(0.4e-9) * (F(3.74183e-16) * (F(1) / p5))
    return num / (F(math.exp(float(F(1.4388e-2) / (w1 * F(temp))))) - F(1))


def spectrum_blackbody(temp) -> np.ndarray:
    """sBlackBody (Spectrum.hs:480-483): fromSpd of an SpdFunc, each band the
    mean of the function at the band's two edges (avgSpd, :316).  The
    exponential is evaluated in double and rounded once, a stand-in for GHC's
    expf."""
    out = []
    for i in range(BANDS):
        l0 = lerp(F(i) / F(BANDS), LAMBDA_START, LAMBDA_END)
        l1 = lerp(F(i + 1) / F(BANDS), LAMBDA_START, LAMBDA_END)
        out.append((_planck(temp, l0) + _planck(temp, l1)) * F(0.5))
    return np.asarray(out, np.float32)


# ---------------------------------------------------------------- the parser
class _State:
    """PState with the reference's start values (RenderJob.hs:24-33)."""

    def __init__(self, base: Path):
        self.res = (640, 480)
        self.renderer = "path"
        self.photons = 0  # photons per pass of the light tracer
        self.sppm = None  # mkSPPM arguments
        self.sampler = (abi.SAMPLER_STRATIFIED, (2, 2))
        self.depths = (7, 3)
        self.filter = (abi.FILTER_BOX, (0.0, 0.0, 0.0, 0.0))
        # defaultCamera 640 480 (CameraParser.hs): fixed at 640 x 480
        self.camera = (xf.translate(0, 0, -5), F(0), F(1), F(90), 640, 480)
        self.transform = xf.identity()
        self.material = None  # defaultMaterial, created on first use
        self.emit = None
        self.lights = []      # newest first
        self.blocks = []      # primitive blocks, newest first: ("mesh", i) / ("shape", i)
        self.base = base


class _Parser:
    def __init__(self, text: str, base: Path):
        self.t = _Tokens(text)
        self.s = _State(base)
        self.scene = Scene()

    # -- state ---------------------------------------------------------
    def _material(self) -> int:
        if self.s.material is None:  # mkMatte (rgbR 0.9 0.9 0.9) 0 (MaterialParser.hs)
            self.s.material = self.scene.add_material(
                abi.MAT_MATTE, kd=rgb_to_spectrum((F(0.9), F(0.9), F(0.9))), sigma=0.0)
        return self.s.material

    # -- job -----------------------------------------------------------
    def job(self) -> Job:
        t = self.t
        while t.peek()[0] is not None:
            name = t.word()
            handler = {
                "filter": self.p_filter, "prim": self.p_prim, "imageSize": self.p_size,
                "renderer": self.p_renderer, "transform": self.p_global_trans,
                "newTransform": self.p_new_transform, "camera": self.p_camera,
                "light": self.p_light, "material": self.p_material,
                "emission": self.p_emission,
            }.get(name)
            if handler is None:
                raise t.error(f"unknown object type {name}")
            handler()
        sc = self.scene
        self._material()  # a file without prims still has the default material
        sc.prim_order = [v if k == "mesh" else ~v for k, v in self.s.blocks]
        sc.lights = list(self.s.lights)
        c2w, lr, fd, fov, sx, sy = self.s.camera
        sc.set_perspective(c2w, float(lr), float(fd), fov, sx, sy)
        (kind, strata), (md, sd) = self.s.sampler, self.s.depths
        fk, fp = self.s.filter
        return Job(sc, self.s.res[0], self.s.res[1], fk, fp, self.s.renderer, kind, strata, md, sd,
                   self.s.photons, self.s.sppm, (c2w, float(lr), float(fd), fov))

    def p_size(self):
        self.s.res = (self.t.integ(), self.t.integ())

    def p_filter(self):
        t = self.t
        name = t.word()
        if name == "box":
            self.s.filter = (abi.FILTER_BOX, (0.0, 0.0, 0.0, 0.0))
        elif name == "gauss":
            self.s.filter = (abi.FILTER_GAUSS, (t.flt(), t.flt(), t.flt(), 0.0))
        elif name == "sinc":
            self.s.filter = (abi.FILTER_SINC, (t.flt(), t.flt(), t.flt(), 0.0))
        elif name == "triangle":
            self.s.filter = (abi.FILTER_TRIANGLE, (t.flt(), t.flt(), 0.0, 0.0))
        elif name == "mitchell":
            self.s.filter = (abi.FILTER_MITCHELL, (t.flt(), t.flt(), t.flt(), t.flt()))
        else:
            raise t.error(f'unknown pixel filter function "{name}"')

    # -- renderer (RendererParser.hs, IntegratorParser.hs) --------------
    def p_renderer(self):
        t = self.t

        def body():
            name = t.word()
            if name == "light":  # mkLightTracer ppp, run by bling_light_pass
                self.s.photons = t.named_int("passPhotons")
                self.s.renderer = "light"
                return
            if name == "sppm":  # mkSPPM n md r alpha, run by bling_sppm_pass
                n, md = t.named_int("photonCount"), t.named_int("maxDepth")
                r = t.named_flt("radius")
                a = t.named_flt("alpha") if t.at("alpha") else F(0.8)
                self.s.sppm = (n, md, r, a)
                self.s.renderer = "sppm"
                return
            if name != "sampler":
                self._skip_to_block_end()
                self.s.renderer = name
                return
            sampler, depths = t.named_block("sampled", self._sampled)
            self.s.sampler = sampler
            if depths is None:
                return
            self.s.depths = depths
            self.s.renderer = "path"
        t.block(body)

    def _sampled(self):
        t = self.t

        def sampler():
            kind = t.word()
            if kind == "stratified":
                return (abi.SAMPLER_STRATIFIED, (t.integ(), t.integ()))
            if kind == "random":
                return (abi.SAMPLER_RANDOM, (t.integ(), 1))
            raise t.error(f"unknown sampler type {kind}")
        smp = t.named_block("sampler", sampler)

        def integrator():
            kind = t.word()
            if kind == "path":
                return (t.named_int("maxDepth"), t.named_int("sampleDepth"))
            self._skip_to_block_end()
            self.s.renderer = f"sampler/{kind}"
            return None
        depths = t.named_block("integrator", integrator)
        return smp, depths

    def _skip_to_block_end(self):
        """consumes tokens up to (not including) the '}' closing the current block"""
        depth = 0
        while True:
            kind, val, _ = self.t.peek()
            if val is None:
                raise self.t.error("unterminated block")
            if val == "}" and depth == 0:
                return
            self.t.next()
            depth += {"{": 1, "}": -1}.get(val, 0)

    # -- transforms (TransformParser.hs) --------------------------------
    def p_transform(self) -> xf.Transform:
        t = self.t

        def body():
            ts = []
            while not t.at("}"):
                name = t.word()
                if name == "rotateX":
                    ts.append(xf.rotate_x(t.flt()))
                elif name == "rotateY":
                    ts.append(xf.rotate_y(t.flt()))
                elif name == "rotateZ":
                    ts.append(xf.rotate_z(t.flt()))
                elif name == "scale":
                    ts.append(xf.scale(*t.vec()))
                elif name == "translate":
                    ts.append(xf.translate(*t.vec()))
                elif name == "matrix":
                    ts.append(t.block(self._matrix))
                elif name == "lookAt":
                    ts.append(t.block(lambda: xf.look_at(t.named_vec("pos"), t.named_vec("look"),
                                                         t.named_vec("up"))))
                else:
                    raise t.error(f"unknown transform {name}")
            # mconcat = foldr (<>) mempty
            acc = xf.identity()
            for tr in reversed(ts):
                acc = xf.concat(tr, acc)
            return acc
        return t.block(body)

    def _matrix(self):
        t = self.t
        rows = []
        for _ in range(4):
            t.expect("m")
            rows.append([t.flt() for _ in range(4)])
        m = np.asarray(rows, np.float32).reshape(16)
        return xf.Transform(m, xf.invert(m))

    def p_global_trans(self):
        self.s.transform = xf.concat(self.p_transform(), self.s.transform)

    def p_new_transform(self):
        self.s.transform = xf.identity()
        self.p_global_trans()

    # -- camera (CameraParser.hs) ---------------------------------------
    def p_camera(self):
        t = self.t

        def body():
            kind = t.word()
            if kind != "perspective":
                raise Unsupported(f"camera {kind}: the GPU path renders perspective cameras")
            fov = t.named_flt("fov")
            lr = t.named_flt("lensRadius")
            fd = t.named_flt("focalDistance")
            sx, sy = self.s.res
            self.s.camera = (self.s.transform, lr, fd, fov, sx, sy)
        t.block(body)

    # -- spectra (ParserCore.hs:151-190) --------------------------------
    def p_spectrum(self) -> np.ndarray:
        t = self.t
        kind = t.word()
        if kind in ("rgbR", "rgbI"):
            rgb = self._rgb()
            return rgb_to_spectrum(rgb, illuminant=(kind == "rgbI"))
        if kind == "spd":
            def body():
                pairs = [(t.flt(), t.flt())]
                while t.at(","):
                    t.next()
                    pairs.append((t.flt(), t.flt()))
                return pairs
            return spectrum_from_spd(t.block(body))
        if kind == "temp":
            return spectrum_blackbody(t.flt())
        raise t.error(f"unknown spectrum type {kind}")

    def _rgb(self):
        kind, val, line = self.t.peek()
        if kind == "hex":
            self.t.next()
            digits = val[1:].replace(" ", "").replace("\t", "").replace("\n", "")
            return tuple(F(int(digits[k:k + 2], 16)) / F(255) for k in (0, 2, 4))
        return (self.t.flt(), self.t.flt(), self.t.flt())

    # -- materials (MaterialParser.hs) ----------------------------------
    # A texture parses to its constant (a spectrum or a float) when it is
    # `constant`, else to a _Node: a node of the scene's texture expressions.
    def _spectrum_texture(self, name):
        """pSpectrumTexture name (MaterialParser.hs:202-226)"""
        t = self.t
        sc = self.scene

        def body():
            kind = t.word()
            if kind == "constant":
                return self.p_spectrum()
            if kind == "blend":  # spectrumBlend tex1 tex2 f
                a = self._spectrum_texture("tex1")
                b = self._spectrum_texture("tex2")
                f = self._scalar_texture("f")
                return _Node(sc.tex_blend(self._snode(a), self._snode(b), self._fnode(f)))
            if kind == "image":
                px, mapping = t.block(lambda: self._image(rgb=True))
                return _Node(sc.tex_image(px, mapping))
            if kind == "checker":
                scale = tuple(t.vec())
                a = self._spectrum_texture("tex1")
                b = self._spectrum_texture("tex2")
                return _Node(sc.tex_checker(scale, self._snode(a), self._snode(b)))
            if kind == "gradient":
                f = self._scalar_texture("f")
                steps = t.named_block("steps", self._gradient_steps)
                return _Node(sc.tex_gradient(steps, self._fnode(f)))
            if kind == "graphPaper":
                lw = t.flt()
                mapping = self._mapping2d("map")
                a = self._spectrum_texture("tex1")
                b = self._spectrum_texture("tex2")
                return _Node(sc.tex_graph_paper(lw, mapping, self._snode(a), self._snode(b)))
            raise t.error(f"unknown texture type {kind}")
        return t.named_block(name, body)

    def _scalar_texture(self, name):
        """pScalarTexture name (MaterialParser.hs:120-163)"""
        t = self.t
        sc = self.scene

        def body():
            kind = t.word()
            if kind == "constant":
                return t.flt()
            if kind == "image":
                px, mapping = t.block(lambda: self._image(rgb=False))
                return _Node(sc.tex_image_scalar(px, mapping))
            if kind == "cellNoise":
                dname = t.word()
                dists = {"euclidian": abi.DIST_EUCLIDIAN, "euclidian2": abi.DIST_EUCLIDIAN2,
                         "manhattan": abi.DIST_MANHATTAN, "chebyshev": abi.DIST_CHEBYSHEV}
                if dname not in dists:
                    raise t.error(f"unknown distance function {dname}")
                return _Node(sc.tex_cell_noise(dists[dname], self._mapping3d("map")))
            if kind == "fbm":
                octaves = t.named_int("octaves")
                omega = t.named_flt("omega")
                return _Node(sc.tex_fbm(octaves, omega, self._mapping3d("map")))
            if kind == "perlin":
                return _Node(sc.tex_perlin(self._mapping3d("map")))
            if kind == "crystal":
                octaves = t.named_int("octaves")
                return _Node(sc.tex_crystal(octaves, self._mapping2d("map")))
            if kind == "scale":
                a, f = t.flt(), t.flt()
                tex = self._scalar_texture("tex")
                return _Node(sc.tex_scale(a, f, self._fnode(tex)))
            raise t.error(f"unknown texture type {kind}")
        return t.named_block(name, body)

    def _snode(self, v) -> int:
        """a spectrum texture as a node (a constant becomes one)"""
        return v.index if isinstance(v, _Node) else self.scene.tex_constant(v)

    def _fnode(self, v) -> int:
        return v.index if isinstance(v, _Node) else self.scene.tex_scalar(v)

    def _mapping2d(self, name):
        """pTextureMapping2d (MaterialParser.hs:168-186)"""
        t = self.t

        def body():
            kind = t.word()
            if kind == "planar":
                vu, vv = t.vec(), t.vec()
                return planar_mapping(vu, vv, t.flt(), t.flt())
            if kind == "uv":
                su, sv, ou, ov = t.flt(), t.flt(), t.flt(), t.flt()
                return uv_mapping(su, sv, ou, ov)
            raise t.error(f"unknown 2d mapping {kind}")
        return t.named_block(name, body)

    def _mapping3d(self, name):
        """pTextureMapping3d: identity with its transform (MaterialParser.hs:188-194)"""
        t = self.t

        def body():
            kind = t.word()
            if kind != "identity":
                raise t.error(f"unknown 3d mapping {kind}")
            return identity_mapping(self.p_transform())
        return t.named_block(name, body)

    def _gradient_steps(self):
        """`pos spectrum` pairs separated by commas (MaterialParser.hs:213-218)"""
        steps = []
        t = self.t
        while not t.at("}"):
            pos = t.flt()
            steps.append((pos, self.p_spectrum()))
            if t.at(","):
                t.next()
        return steps

    def _image(self, rgb: bool):
        """`file "name"` and the 2D mapping: readImageTextureMap (8-bit RGB,
        RGBA with the alpha dropped) or readImageScalarMap (8-bit grey)
        (Texture.hs:110-126).  PNG files only."""
        t = self.t
        t.expect("file")
        kind, val, line = t.next()
        if kind != "str":
            raise BlingFileError(f"line {line}: expected a file name, got {val!r}")
        path = self.s.base / val[1:-1]
        if path.suffix.lower() != ".png":
            raise Unsupported(f"image {path.name}: PNG images are read")
        px = image.read_png(path)
        if rgb:
            if px.ndim == 2 or px.shape[2] not in (3, 4):
                raise BlingFileError(f"line {line}: {path.name}: not an RGB image")
            px = px[..., :3]
        elif px.ndim != 2:
            raise BlingFileError(f"line {line}: {path.name}: not a grey image")
        return px, self._mapping2d("map")

    def p_material(self):
        self.s.material = self.t.block(self._material_body)

    def _material_body(self, bump=None) -> int:
        """pMaterial' (MaterialParser.hs:28-40); `bump` the displacement node
        of an enclosing bumpMap"""
        t = self.t
        kind = t.word()
        sc = self.scene
        tex = {}

        def val(v, slot, default):
            """the constant of a parameter, or its node in tex"""
            if isinstance(v, _Node):
                tex[slot] = v.index
                return default
            return v

        def spec(name, slot):
            return val(self._spectrum_texture(name), slot, None)

        def flt(name, slot):
            return float(val(self._scalar_texture(name), slot, 0.0))

        def add(mkind, **kw):
            return sc.add_material(mkind, tex=tex, bump=bump, **kw)
        if kind == "bumpMap":  # pBumpMap: bumpMapped d m (MaterialParser.hs:42-46)
            if bump is not None:
                raise Unsupported("material bumpMap of a bumpMap: one displacement per material")
            d = self._scalar_texture("bump")
            return self._material_body(bump=self._fnode(d))
        if kind == "matte":
            kd = spec("kd", "kd")
            return add(abi.MAT_MATTE, kd=kd, sigma=flt("sigma", "sigma"))
        if kind == "plastic":
            kd = spec("kd", "kd")
            ks = spec("ks", "ks")
            return add(abi.MAT_PLASTIC, kd=kd, ks=ks, roughness=flt("rough", "roughness"))
        if kind == "metal":
            eta = spec("eta", "eta")
            k = spec("k", "k")
            return add(abi.MAT_METAL, eta=eta, k=k, roughness=flt("rough", "roughness"))
        if kind == "glass":
            ior = self._scalar_texture("ior")
            kr = spec("kr", "ks")
            kt = spec("kt", "kt")
            return add(abi.MAT_GLASS, ks=kr, kt=kt, ior=float(val(ior, "ior", 1.5)))
        if kind == "mirror":
            return add(abi.MAT_MIRROR, ks=spec("kr", "ks"))
        if kind == "shinyMetal":
            kr = spec("kr", "kd")
            ks = spec("ks", "ks")
            return add(abi.MAT_SHINY_METAL, kd=kr, ks=ks, roughness=flt("rough", "roughness"))
        if kind == "transMatte":
            kr = spec("kr", "kd")
            kt = spec("kt", "kt")
            return add(abi.MAT_TRANS_MATTE, kd=kr, kt=kt, sigma=flt("ks", "sigma"))
        if kind == "substrate":  # pSubstrateMaterial (MaterialParser.hs:50-58)
            kd = spec("kd", "kd")
            ks = spec("ks", "ks")
            ka = spec("ka", "kt")
            ur = flt("urough", "roughness")
            vr = flt("vrough", "sigma")
            depth = flt("depth", "ior")
            return add(abi.MAT_SUBSTRATE, kd=kd, ks=ks, kt=ka, roughness=ur, sigma=vr, ior=depth)
        if kind == "blackbody":
            return add(abi.MAT_BLACKBODY)
        raise t.error(f"unknown material type {kind}")

    def p_emission(self):
        t = self.t

        def body():
            if t.at("none"):
                t.next()
                return None
            return self.p_spectrum()
        self.s.emit = t.block(body)

    # -- lights (LightParser.hs) ----------------------------------------
    def p_light(self):
        t = self.t

        def body():
            kind = t.word()
            if kind == "directional":
                t.expect("intensity")
                s = self.p_spectrum()
                n = xf.normalize(t.named_vec("normal"))
                return Light(abi.LIGHT_DIRECTIONAL, s, vec=tuple(float(x) for x in n))
            if kind == "point":
                t.expect("intensity")
                s = self.p_spectrum()
                p = t.named_vec("position")
                return Light(abi.LIGHT_POINT, s, vec=tuple(float(x) for x in p))
            if kind == "infinite":
                w2l = self.p_transform()
                t.expect("l")
                env = t.block(self._env_map)
                if isinstance(env, dict):  # mkSunSkyLight east sunDir turbidity
                    return Light(abi.LIGHT_SUNSKY, vec=env["sunDir"], east=env["east"],
                                 turbidity=env["turbidity"], w2l=w2l)
                return Light(abi.LIGHT_INFINITE, env=env, w2l=w2l)
            raise t.error(f"unknown light type {kind}")
        self.s.lights.insert(0, t.block(body))

    def _env_map(self):
        t = self.t
        kind = t.word()
        if kind == "constant":  # constSpectrumMap2d: a 1 x 1 map (Texture.hs:131-132)
            return self.p_spectrum().reshape(1, 1, BANDS)
        if kind == "sunSky":  # MaterialParser.hs:266-270
            east = tuple(float(x) for x in t.named_vec("east"))
            sun = tuple(float(x) for x in t.named_vec("sunDir"))
            return {"east": east, "sunDir": sun, "turbidity": float(t.named_flt("turbidity"))}
        if kind in ("file", "rgbeFile"):
            raise Unsupported(f"environment map {kind}: the GPU path takes constant maps from "
                              ".bling files (image maps through bling_light_desc.env)")
        raise t.error(f"unknown map type {kind}")

    # -- primitives (PrimitiveParser.hs) --------------------------------
    def p_prim(self):
        self.t.block(self._prim_body)

    def _prim_body(self):
        t = self.t
        kind = t.word()
        if kind == "mesh":
            self._mesh()
        elif kind == "shape":
            self._shape()
        elif kind == "heightMap":
            self._height_map()
        elif kind == "waveFront":
            self._wave_front()
        elif kind in ("bezier", "julia", "mandelbulb"):
            raise Unsupported(f"primitive {kind}: the GPU path renders meshes and shapes")
        else:
            raise t.error(f"unknown primitive type {kind}")

    def _mesh(self):
        """pMesh + mkTriangleMesh: vertices moved to world space with
        transPoint at build (TriangleMesh.hs:58), faces fanned (triangulate)."""
        t = self.t
        vc = t.named_int("vertexCount")
        fc = t.named_int("faceCount")
        verts = []
        for _ in range(vc):
            t.expect("v")
            verts.append(trans_point(self.s.transform, t.vec()))
        idx = []
        for _ in range(fc):
            t.expect("f")
            face = [t.integ()]
            while t.peek()[0] == "num":
                face.append(t.integ())
            for k in range(1, len(face) - 1):
                idx += [face[0], face[k], face[k + 1]]
        v = np.asarray(verts, np.float32).reshape(-1, 3)
        m = self.scene.add_mesh(v, np.asarray(idx, np.int32), self._material())
        self.s.blocks.insert(0, ("mesh", m))

    # -- scalar maps for heightMap (pScalarMap2d, MaterialParser.hs:228-245)
    def _scalar_map2d(self):
        """a function of float32 arrays (x, y) -> elevation"""
        t = self.t

        def body():
            kind = t.word()
            if kind == "fbm":  # texMap3dTo2d (fbm octaves omega) z
                z = t.flt()
                octaves = t.named_int("octaves")
                omega = t.named_flt("omega")
                return lambda x, y: noise.fbm(octaves, omega, x, y, np.full_like(x, z))
            if kind == "scale":
                f = t.flt()
                m = self._scalar_map2d()
                return lambda x, y: F(f) * m(x, y)
            raise t.error(f"unknown scalar map type{kind}")
        return t.block(body)

    def _height_map(self):
        """heightMap ns nt elevation transform (PrimitiveParser.hs:39-45,
        Heightmap.hs:15-49): an ns x nt grid over [0, 1]^2 lifted by the
        elevation, shading normals from central differences, uvs, built with
        mkTriangleMesh in the given transform"""
        t = self.t
        ns, nt = t.integ(), t.integ()
        elev = self._scalar_map2d()
        tr = self.p_transform()
        fns, fnt = F(ns), F(nt)
        xs = np.arange(ns, dtype=F) / (fns - F(1))
        zs = np.arange(nt, dtype=F) / (fnt - F(1))
        X, Z = np.meshgrid(xs, zs)  # [z, x]: coords z-major, as the comprehension
        X, Z = X.reshape(-1), Z.reshape(-1)
        pts = np.stack([X, elev(X, Z), Z], -1)
        ex, ez = F(1) / fns, F(1) / fnt
        dx = elev(X - ex, Z) - elev(X + ex, Z)
        dz = elev(X, Z - ez) - elev(X, Z + ez)
        nrm = -_normalize_rows(np.stack([dx, np.full_like(dx, ex + ez), dz], -1))
        uvs = np.stack([X / (fns - F(1)), Z / (fns - F(1))], -1)  # both over ns - 1
        x, y = np.meshgrid(np.arange(ns - 1), np.arange(nt - 1))
        x, y = x.reshape(-1), y.reshape(-1)
        v = lambda a, b: a + b * ns  # noqa: E731
        idx = np.stack([v(x, y), v(x + 1, y), v(x + 1, y + 1),
                        v(x, y), v(x + 1, y + 1), v(x, y + 1)], -1).reshape(-1)
        m = self.scene.add_mesh(_trans_points(tr, pts), idx.astype(np.int32), self._material(),
                                normals=_trans_normals(tr, nrm), uvs=uvs)
        self.s.blocks.insert(0, ("mesh", m))

    def _wave_front(self):
        """waveFront "file" materials { "name" { material } ... }
        (PrimitiveParser.hs:69-72, IO/WaveFront.hs): the file's faces fanned
        into triangles, grouped by `usemtl` into runs of one material (names
        missing from the map take the current material), vertices moved by
        the current transform.  Every triangle keeps its own corners' uvs and
        normals, so the corners become vertices of their own; as the
        reference reads them, a triangle's third corner takes the uv and
        normal indices of its second, normals are not transformed, and the
        last run is cut to the face count less its starting corner index."""
        t = self.t
        kind, val, line = t.next()
        if kind != "str":
            raise BlingFileError(f"line {line}: expected a file name, got {val!r}")
        path = self.s.base / val[1:-1]
        t.expect("materials")

        def body():
            mats = {}
            while not t.at("}"):
                k, name, ln = t.next()
                if k != "str":
                    raise BlingFileError(f"line {ln}: expected a material name, got {name!r}")
                mats[name[1:-1]] = t.block(self._material_body)
            return mats
        mats = t.block(body)
        obj = _read_obj(path)
        default = self._material()
        P = _trans_points(self.s.transform, obj["v"]) if len(obj["v"]) else obj["v"]
        corners = obj["corners"]  # (n, 3): point, uv, normal index per face corner, 0-based
        n_tri = len(corners) // 3
        # matIntervals: runs from each usemtl's corner count; the last one ends
        # at the triangle count (WaveFront.hs:95-99, 111)
        starts = [("default", 0)] + obj["mtls"]
        ends = [c for _, c in obj["mtls"]] + [n_tri]
        meshes = []
        for (name, s0), e in zip(starts, ends):
            if e - s0 <= 0:
                continue
            tris = list(range(s0, s0 + (e - s0), 3))  # [s, s+3 .. s+l-1], corner indices
            tris = [i for i in tris if i + 2 < len(corners)]
            if not tris:
                continue
            mat = mats.get(name, default)
            meshes += _obj_meshes(P, obj["vn"], obj["vt"], corners, tris, mat)
        for mesh in meshes:
            m = self.scene.add_mesh(*mesh)
            self.s.blocks.insert(0, ("mesh", m))
        # blocks are newest first: this primitive's meshes in their own order
        k = len(meshes)
        self.s.blocks[:k] = self.s.blocks[:k][::-1]

    def _shape(self):
        t = self.t

        def body():
            kind = t.word()
            if kind == "box":  # mkBox (Shape.hs:41-44)
                a, b = t.named_vec("pmin"), t.named_vec("pmax")
                lo = [_ghc_min(a[k], b[k]) for k in range(3)]
                hi = [_ghc_max(a[k], b[k]) for k in range(3)]
                return abi.SHAPE_BOX, tuple(lo + hi)
            if kind == "cylinder":  # mkCylinder (Shape.hs:47-56)
                r = t.named_flt("radius")
                z0, z1 = t.named_flt("zmin"), t.named_flt("zmax")
                pm = xf.radians(_clamp(t.named_flt("phiMax"), F(0), F(360)))
                return abi.SHAPE_CYLINDER, (r, _ghc_min(z0, z1), _ghc_max(z0, z1), pm)
            if kind == "disk":  # mkDisk (Shape.hs:59-68)
                h = t.named_flt("height")
                r0, r1 = t.named_flt("radius"), t.named_flt("innerRadius")
                pm = xf.radians(_clamp(t.named_flt("phiMax"), F(0), F(360)))
                return abi.SHAPE_DISK, (h, _ghc_max(r0, r1), _ghc_min(r0, r1), pm)
            if kind == "quad":
                return abi.SHAPE_QUAD, (t.flt(), t.flt())
            if kind == "sphere":
                return abi.SHAPE_SPHERE, (t.named_flt("radius"),)
            raise t.error(f"unknown shape type {kind}")
        kind, params = t.block(body)
        # mkGeom (transform s) False (material s) (emit s) shp sid
        sh = self.scene.add_shape(kind, tuple(float(p) for p in params), self.s.transform,
                                  self._material(), emission=self.s.emit)
        self.s.blocks.insert(0, ("shape", sh))


def _trans_points(t: xf.Transform, p) -> np.ndarray:
    """trans_point of an (n, 3) array, float32, same operation order"""
    m = [F(x) for x in t.m]
    x, y, z = (np.asarray(p[:, k], F) for k in range(3))

    def row(r):
        return ((m[4 * r] * x + m[4 * r + 1] * y) + m[4 * r + 2] * z) + m[4 * r + 3]
    xp, yp, zp, wp = row(0), row(1), row(2), row(3)
    one = wp == F(1)
    out = np.stack([np.where(one, xp, xp / wp), np.where(one, yp, yp / wp),
                    np.where(one, zp, zp / wp)], -1)
    return out.astype(F)


def _trans_normals(t: xf.Transform, n) -> np.ndarray:
    """transNormal (Transform.hs:266-272) of an (n, 3) array: the transposed
    inverse, float32"""
    mi = [F(x) for x in t.inv]
    x, y, z = (np.asarray(n[:, k], F) for k in range(3))
    return np.stack([(mi[0] * x + mi[4] * y) + mi[8] * z, (mi[1] * x + mi[5] * y) + mi[9] * z,
                     (mi[2] * x + mi[6] * y) + mi[10] * z], -1).astype(F)


def _normalize_rows(v) -> np.ndarray:
    """normalize (Math.hs:349-353) of each row, float32"""
    v = np.asarray(v, F)
    sl = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]
    il = F(1) / np.sqrt(np.where(sl != 0, sl, F(1)))
    out = v * il[:, None]
    out[sl == 0] = (0, 1, 0)
    return out.astype(F)


def _read_obj(path: Path) -> dict:
    """The lines of a Wavefront .obj file that waveFrontParser reads
    (IO/WaveFront.hs:128-211): v, vn (normalised), vt (v defaults to 1), f
    (fanned; point/uv/normal indices 1-based, a missing one 0, so -1 here),
    usemtl (the material's name and the corner count so far); other lines
    are skipped"""
    v, vn, vt, corners, mtls = [], [], [], [], []
    for raw in path.read_text().splitlines():
        parts = raw.split()
        if not parts:
            continue
        key = parts[0]
        if key == "v":
            v.append([f32_of_decimal(x) for x in parts[1:4]])
        elif key == "vn":
            vn.append([f32_of_decimal(x) for x in parts[1:4]])
        elif key == "vt":
            vt.append((f32_of_decimal(parts[1]),
                       f32_of_decimal(parts[2]) if len(parts) > 2 else F(1)))
        elif key == "f":
            idx = []
            for tok in parts[1:]:
                fs = tok.split("/")
                p = int(fs[0])
                uv = int(fs[1]) if len(fs) > 1 and fs[1] else 0
                nn = int(fs[2]) if len(fs) > 2 and fs[2] else 0
                idx.append((p - 1, uv - 1, nn - 1))
            for k in range(1, len(idx) - 1):  # triangulate: a fan
                corners += [idx[0], idx[k], idx[k + 1]]
        elif key == "usemtl":
            mtls.append((raw.split(None, 1)[1].strip() if len(parts) > 1 else "", len(corners)))
    vn_arr = _normalize_rows(np.asarray(vn, F).reshape(-1, 3)) if vn else np.zeros((0, 3), F)
    return {"v": np.asarray(v, F).reshape(-1, 3), "vn": vn_arr, "vt": np.asarray(vt, F).reshape(-1, 2),
            "corners": np.asarray(corners, np.int64).reshape(-1, 3), "mtls": mtls}


def _obj_meshes(P, VN, VT, corners, tris, mat):
    """the triangles at corner indices `tris` (one run of a material) as
    meshes of three vertices per triangle, split where the presence of
    normals changes (a mesh has normals for all its vertices or none)"""
    out = []
    run = []

    def flush():
        if not run:
            return
        has_n = run[0][1]
        verts, nrm, uvs = [], [], []
        for i, _ in run:
            c = corners[i:i + 3]
            # wfTriUVs / wfTriNormals: corners i, i+1 and i+1 (WaveFront.hs:51-76)
            ui = (c[0][1], c[1][1], c[1][1])
            ni = (c[0][2], c[1][2], c[1][2])
            verts += [P[c[0][0]], P[c[1][0]], P[c[2][0]]]
            if min(ui) >= 0:
                uvs += [VT[ui[0]], VT[ui[1]], VT[ui[2]]]
            else:  # triangleDefaultUVs
                uvs += [(0, 0), (1, 0), (1, 1)]
            if has_n:
                nrm += [VN[ni[0]], VN[ni[1]], VN[ni[2]]]
        k = len(run)
        out.append((np.asarray(verts, F).reshape(-1, 3), np.arange(3 * k, dtype=np.int32), mat,
                    np.asarray(nrm, F).reshape(-1, 3) if has_n else None,
                    np.asarray(uvs, F).reshape(-1, 2)))
        run.clear()
    for i in tris:
        c = corners[i:i + 3]
        ni = (c[0][2], c[1][2], c[1][2])
        if max(ni) < 0:
            has_n = False
        elif min(ni) >= 0:
            has_n = True
        else:
            raise BlingFileError("a face gives normals for some corners only")
        if run and run[0][1] != has_n:
            flush()
        run.append((i, has_n))
    flush()
    return out


def parse(text: str, base_path: str | Path = ".") -> Job:
    """Parses .bling source text (parseJob, RenderJob.hs:36-48)."""
    return _Parser(text, Path(base_path)).job()


def load(path: str | Path) -> Job:
    """Reads and parses a .bling file; relative resources resolve against its
    directory."""
    p = Path(path)
    return parse(p.read_text(), p.parent)
