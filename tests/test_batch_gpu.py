"""The batched job engine on the GPU (bling_batch_*).

Every sample's random numbers depend only on its job's seed and pass and on
its pixel and sample number, and the per-vertex arithmetic is the same code
as bling_render_pass's, so a job renders the same film in a batch as alone.
Only the order of the float additions into the film differs (atomics), so:

* film weights are equal exactly (box filter: sums of 1.0);
* film XYZ agree within 1e-5 relative (plus 1e-6 of the film's largest value);
* ray counts and path-sample counts are equal exactly.
"""
import numpy as np
import pytest

from bling_gb300 import abi
from bling_gb300 import scene as S
from bling_gb300.api import Batch, BlingError, Context

pytestmark = pytest.mark.gpu


def _same(fa, fb, exact_weights=True):
    if exact_weights:
        assert np.array_equal(fa[..., 0], fb[..., 0]), "film weights differ"
    else:
        assert np.allclose(fa[..., 0], fb[..., 0], rtol=1e-5, atol=1e-6)
    scale = float(np.abs(fb[..., 1:]).max()) + 1e-30
    assert np.allclose(fa[..., 1:], fb[..., 1:], rtol=1e-5, atol=1e-6 * scale), (
        float(np.abs(fa[..., 1:] - fb[..., 1:]).max()), scale)


def _alone(ctx, g, params, pass_index):
    """a job rendered alone by bling_render_pass: film and counters"""
    film = ctx.film(params.width, params.height)
    before = g.stats()
    g.render_pass(film, params, pass_index)
    after = g.stats()
    counts = {k: after[k] - before[k] for k in ("rays_closest", "rays_any", "path_samples")}
    return film.read(), counts


def _jobs(ctx):
    """scenes of different kinds and sizes and jobs of different image sizes,
    sample counts, depths, filters and passes (two jobs share a scene)"""
    cornell = S.cornell_room(48, 40)
    soup = S.soup_spheres_scene(20000, n_spheres=64, seed=5, width=56, height=56)
    hf = S.heightfield_scene(ns=129, n_spheres=64, width=64, height=36, env_size=(64, 32))
    g_c, g_s, g_h = ctx.scene(cornell), ctx.scene(soup), ctx.scene(hf)
    jobs = [
        (g_c, S.cornell_params(48, 40, spp_side=2, max_depth=5, rr_depth=3, seed=3), 0),
        (g_s, S.render_params(56, 56, (3, 2), max_depth=7, sample_depth=3, rr_depth=3, seed=9), 1),
        (g_h, S.render_params(64, 36, (2, 2), max_depth=8, sample_depth=3, rr_depth=3,
                              filter_kind=abi.FILTER_MITCHELL,
                              filter_params=(2, 2, 1 / 3, 1 / 3), seed=4), 0),
        (g_c, S.cornell_params(48, 40, spp_side=3, max_depth=3, rr_depth=1, seed=5), 7),
        (g_s, S.render_params(56, 56, (1, 1), max_depth=10, sample_depth=2, rr_depth=2, seed=2), 2),
    ]
    return jobs


@pytest.mark.parametrize("mode,sort_rays", [(abi.BATCH_PLAIN_LAUNCHES, False),
                                            (abi.BATCH_GRAPH, False),
                                            (abi.BATCH_GRAPH, True),
                                            (abi.BATCH_DEVICE_LOOP, False),
                                            (abi.BATCH_DEVICE_LOOP, True)])
def test_each_job_renders_the_same_alone_and_in_the_mix(gpu_ctx, mode, sort_rays):
    jobs = _jobs(gpu_ctx)
    # few slots: paths of all jobs share the queues and slots are reused many times
    b = Batch(gpu_ctx, slots=4096, graph_mode=mode, sort_rays=sort_rays, iters_per_launch=8)
    films, ids = [], []
    for g, p, k in jobs:
        f = gpu_ctx.film(p.width, p.height)
        films.append(f)
        ids.append(b.submit(g, f, p, k))
    b.run()
    st = b.stats()
    tot = {"rays_closest": 0, "rays_any": 0, "path_samples": 0}
    for (g, p, k), f, j in zip(jobs, films, ids):
        ref, counts = _alone(gpu_ctx, g, p, k)
        _same(f.read(), ref, exact_weights=p.filter_kind == abi.FILTER_BOX)
        d, t = b.status(j)
        assert d == t == counts["path_samples"]
        for key in tot:
            tot[key] += counts[key]
    assert st["path_samples"] == tot["path_samples"] == st["samples_submitted"]
    assert st["rays_closest"] == tot["rays_closest"]
    assert st["rays_any"] == tot["rays_any"]
    assert st["jobs_done"] == len(jobs) and st["jobs_active"] == 0
    b.close()


def test_jobs_submitted_while_others_run(gpu_ctx):
    """continuous batching: jobs join between steps and each still renders
    what it renders alone"""
    jobs = _jobs(gpu_ctx)
    b = Batch(gpu_ctx, slots=2048, graph_mode=abi.BATCH_GRAPH)
    films, ids = [], []
    g, p, k = jobs[1]
    films.append(gpu_ctx.film(p.width, p.height))
    ids.append(b.submit(g, films[0], p, k))
    b.step(3)
    d0, t0 = b.status(ids[0])
    assert 0 < d0 < t0  # in flight
    for g, p, k in jobs[2:]:
        f = gpu_ctx.film(p.width, p.height)
        films.append(f)
        ids.append(b.submit(g, f, p, k))
        b.step(2)
    b.run()
    for (g, p, k), f, j in zip(jobs[1:], films, ids):
        ref, _ = _alone(gpu_ctx, g, p, k)
        _same(f.read(), ref, exact_weights=p.filter_kind == abi.FILTER_BOX)
        assert b.done(j)
    b.close()


def test_per_job_camera(gpu_ctx):
    """a job at another image size than the scene's camera passes its own
    camera; it matches a scene whose camera was built for that size"""
    sc = S.soup_spheres_scene(5000, n_spheres=16, seed=8, width=40, height=40)
    g40 = gpu_ctx.scene(sc)
    sc72 = S.soup_spheres_scene(5000, n_spheres=16, seed=8, width=72, height=48)
    g72 = gpu_ctx.scene(sc72)
    p = S.render_params(72, 48, (2, 2), max_depth=5, sample_depth=3, rr_depth=3, seed=6)
    b = Batch(gpu_ctx, slots=4096)
    f = gpu_ctx.film(72, 48)
    b.submit(g40, f, p, 0, camera=sc.camera_for(72, 48))
    b.run()
    ref, _ = _alone(gpu_ctx, g72, p, 0)
    _same(f.read(), ref)
    b.close()


def test_job_table_capacity_and_validation(gpu_ctx):
    sc = S.cornell_room(16, 16)
    g = gpu_ctx.scene(sc)
    p = S.cornell_params(16, 16, spp_side=1)
    b = Batch(gpu_ctx, slots=1024, max_jobs=2)
    f = [gpu_ctx.film(16, 16) for _ in range(3)]
    b.submit(g, f[0], p, 0)
    b.submit(g, f[1], p, 1)
    with pytest.raises(BlingError) as e:
        b.submit(g, f[2], p, 2)
    assert e.value.code == abi.BLING_ERR_STATE
    b.run()
    j = b.submit(g, f[2], p, 2)  # room again once the first jobs completed
    b.run()
    assert b.done(j)
    with pytest.raises(BlingError):  # film size does not match the job
        b.submit(g, gpu_ctx.film(8, 8), p, 0)
    with pytest.raises(BlingError):  # scene of another context
        other = Context(device=0)
        try:
            b.submit(other.scene(sc), f[0], p, 0)
        finally:
            other.close()
    with pytest.raises(BlingError):
        Batch(gpu_ctx, block_size=96)
    with pytest.raises(BlingError):
        Batch(gpu_ctx, max_jobs=3)
    b.close()


def test_run_returns_timeout_at_its_iteration_bound_and_continues_later(gpu_ctx):
    """bling_batch_run stops with BLING_ERR_TIMEOUT once max_run_iterations
    iterations ran with work left; the job stays in flight, and stepping on
    completes it with the film the job renders alone."""
    sc = S.cornell_room(48, 48)
    g = gpu_ctx.scene(sc)
    p = S.cornell_params(48, 48, spp_side=4, max_depth=5, rr_depth=3, seed=21)
    b = Batch(gpu_ctx, slots=4096, max_run_iterations=3)
    film = gpu_ctx.film(48, 48)
    job = b.submit(g, film, p, 0)
    with pytest.raises(BlingError) as e:
        b.run()
    assert e.value.code == abi.BLING_ERR_TIMEOUT
    done, total = b.status(job)
    assert 0 < total and done < total
    assert b.stats()["iterations"] == 3
    while not b.done(job):
        b.step(8)
    ref, _ = _alone(gpu_ctx, g, p, 0)
    _same(film.read(), ref)
    b.close()


@pytest.mark.parametrize("mode", [abi.BATCH_GRAPH, abi.BATCH_DEVICE_LOOP])
def test_textured_scene_joins_a_running_batch(gpu_ctx, mode):
    """a batch whose graph was captured for untextured scenes takes the
    textured shading kernel once a scene with textures is registered; every
    job still renders what it renders alone"""
    from texture_scenes import textured_scene
    cornell = gpu_ctx.scene(S.cornell_room(40, 32))
    tex = gpu_ctx.scene(textured_scene(40, 28))
    pc = S.cornell_params(40, 32, spp_side=2, max_depth=5, rr_depth=3, seed=3)
    pt = S.render_params(40, 28, (2, 2), max_depth=5, sample_depth=2, rr_depth=3, seed=6)
    b = Batch(gpu_ctx, slots=2048, graph_mode=mode, iters_per_launch=4)
    fc, ft = gpu_ctx.film(40, 32), gpu_ctx.film(40, 28)
    b.submit(cornell, fc, pc, 0)
    b.step(2)
    b.submit(tex, ft, pt, 1)
    b.run()
    _same(fc.read(), _alone(gpu_ctx, cornell, pc, 0)[0])
    _same(ft.read(), _alone(gpu_ctx, tex, pt, 1)[0])
    b.close()
