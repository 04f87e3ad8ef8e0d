"""The reference's example scenes, as parsed fixtures (tests/golden/examples,
made by tests/golden/make_example_scenes.py from bling's examples/*.bling).

CPU: every fixture loads into the scene record the reader produces, renders
on the oracle, and -- where bling's examples directory is present --
equals what the reader makes of the file today.
GPU: every fixture renders, reduced in size, on the GPU and on the oracle
with the same random numbers, within the render tests' parity bar."""
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
import make_example_scenes as MK  # noqa: E402
import scene_fixture as F  # noqa: E402

from bling_gb300 import abi  # noqa: E402
from bling_gb300 import scene as S  # noqa: E402
from oracle.oracle import OracleScene  # noqa: E402

FIXTURES = F.fixtures()
NAMES = [p.stem for p in FIXTURES]
# scenes with glossy or specular paths, whose paths a last-bit difference of a
# transcendental sends elsewhere more often
GLOSSY = {"bumpmap", "cellnoise", "cornell-box-specular", "cornell-box-underwater", "ducky",
          "glass-torus", "heightmap", "plastic-test", "race", "substrate", "trans-matte"}


def reduced(job, longest=64):
    """the job's render at `longest` pixels on its longer side: its camera
    rebuilt for that size, 2 x 2 strata, depth 5, roulette after 3"""
    k = longest / max(job.width, job.height)
    w, h = max(8, round(job.width * k)), max(8, round(job.height * k))
    job.scene.camera = job.camera_for(w, h)
    p = S.render_params(w, h, (2, 2), max_depth=5, sample_depth=3, rr_depth=3,
                        filter_kind=job.filter_kind, filter_params=job.filter_params, seed=7)
    return p


def test_fixtures_present():
    assert set(NAMES) == set(MK.EXAMPLES)


@pytest.mark.parametrize("name", NAMES)
def test_fixture_renders_on_the_oracle(name):
    job = F.load(GOLDEN / "examples" / f"{name}.npz")
    p = reduced(job, longest=24)
    film, st = OracleScene(job.scene).render_pass(p, 0)
    assert np.isfinite(film).all()
    assert film[..., 2].sum() > 0
    assert st["path_samples"] > 0


def _record(job):
    """the scene record as comparable bytes and arrays"""
    sc = job.scene
    out = [bytes(m) for m in sc.materials]
    for m in sc.meshes:
        out += [m.vertices.tobytes(), m.indices.tobytes(), m.material,
                None if m.normals is None else m.normals.tobytes(),
                None if m.uvs is None else m.uvs.tobytes()]
    for s in sc.shapes:
        out += [s.kind, np.float32(s.params).tobytes(), s.o2w.m.tobytes(), s.o2w.inv.tobytes(),
                s.material, None if s.emission is None else s.emission.tobytes()]
    for lt in sc.lights:
        out += [lt.kind, np.asarray(lt.spectrum, np.float32).tobytes(),
                np.float32(lt.vec).tobytes(), np.float32(lt.east).tobytes(),
                np.float32(lt.turbidity).tobytes(),
                None if lt.w2l is None else lt.w2l.m.tobytes()]
    for t in sc.textures:
        out += [t.kind, tuple(t.children), t.ivalue, t.mapping[0],
                np.float32(t.mapping[1]).tobytes(), np.float32(t.p).tobytes(),
                None if t.spectrum is None else np.float32(t.spectrum).tobytes(),
                None if t.steps is None else np.float32(t.steps).tobytes(),
                None if t.pixels is None else np.asarray(t.pixels, np.uint8).tobytes()]
    out += [list(sc.prim_order), bytes(sc.camera), job.width, job.height, job.filter_kind]
    return out


@pytest.mark.skipif(MK.source_dir() is None, reason="bling's examples directory not present")
@pytest.mark.parametrize("name", NAMES)
def test_fixture_is_what_the_reader_makes_of_the_file(name):
    fixture = F.load(GOLDEN / "examples" / f"{name}.npz")
    fresh = MK.parse_example(MK.source_dir() / f"{name}.bling")
    assert _record(fixture) == _record(fresh)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_example_gpu_vs_oracle(gpu_ctx, name):
    job = F.load(GOLDEN / "examples" / f"{name}.npz")
    p = reduced(job)
    g = gpu_ctx.scene(job.scene)
    film = gpu_ctx.film(p.width, p.height)
    o = OracleScene(job.scene)
    fo = None
    for k in range(2):
        g.render_pass(film, p, k)
        fo, _ = o.render_pass(p, k, fo)
    fg = film.read()
    if job.filter_kind == abi.FILTER_BOX:
        assert np.array_equal(fg[..., 0], fo[..., 0]), "film weights differ"
    else:
        assert np.allclose(fg[..., 0], fo[..., 0], rtol=1e-5, atol=1e-6), "film weights differ"
    rel, frac = (2e-3, 0.9) if name in GLOSSY else (1e-3, 0.97)
    xyz_g, xyz_o = fg[..., 1:], fo[..., 1:]
    scale = np.abs(xyz_o).mean() + 1e-12
    err = np.abs(xyz_g - xyz_o) / (np.abs(xyz_o) + 1e-3 * scale)
    close = (err <= rel).all(-1)
    assert close.mean() >= frac, f"only {close.mean():.4f} of pixels within {rel}"
    m_g, m_o = xyz_g.mean(axis=(0, 1)), xyz_o.mean(axis=(0, 1))
    assert np.all(np.abs(m_g - m_o) <= 5e-3 * np.abs(m_o) + 1e-9), (m_g, m_o)
    assert xyz_o[..., 1].sum() > 0
