"""The render server on the GPU (bling_server_*): continuous batching.

Jobs arrive from another thread while others run; each finished film must be
the one bling_render_pass renders for the job alone (film weights exact with
the box filter, XYZ within 1e-5 relative plus 1e-6 of the film's largest
value: only the order of the film's float additions differs), and admission
must keep the device memory of path state plus admitted films within the
budget."""
import dataclasses
import threading
import time

import numpy as np
import pytest

from bling_gb300 import abi
from bling_gb300 import scene as S
from bling_gb300.api import BlingError, Server

pytestmark = pytest.mark.gpu


def _same(fa, fb):
    assert np.array_equal(fa[..., 0], fb[..., 0]), "film weights differ"
    scale = float(np.abs(fb[..., 1:]).max()) + 1e-30
    assert np.allclose(fa[..., 1:], fb[..., 1:], rtol=1e-5, atol=1e-6 * scale)


def _alone(ctx, sc, params, pass_index):
    """the job rendered alone by bling_render_pass, through a scene whose
    camera was built for the job's image size"""
    own = dataclasses.replace(sc, camera=sc.camera_for(params.width, params.height))
    g = ctx.scene(own)
    f = ctx.film(params.width, params.height)
    g.render_pass(f, params, pass_index)
    out = f.read()
    f.close()
    g.close()
    return out


def _scenes():
    return [S.cornell_room(32, 32),
            S.soup_spheres_scene(30000, n_spheres=64, seed=21, width=32, height=32),
            S.heightfield_scene(ns=129, n_spheres=32, width=32, height=32, env_size=(64, 32))]


def _job_list(n, seed):
    rng = np.random.default_rng(seed)
    jobs = []
    for k in range(n):
        side = int(np.exp(rng.uniform(np.log(16), np.log(80))))
        sx, sy = int(rng.integers(1, 4)), int(rng.integers(1, 4))
        p = S.render_params(side, side + int(rng.integers(0, 9)), (sx, sy),
                            max_depth=int(rng.integers(3, 9)), sample_depth=3, rr_depth=3,
                            seed=int(rng.integers(1, 1 << 30)))
        jobs.append((int(rng.integers(0, 3)), p, int(rng.integers(0, 5))))
    return jobs


def test_jobs_arriving_under_load_render_as_alone(gpu_ctx):
    scenes = _scenes()
    gs = [gpu_ctx.scene(s) for s in scenes]
    jobs = _job_list(14, seed=3)
    srv = Server(gpu_ctx, slots=8192, iters_per_step=2)
    tickets = [None] * len(jobs)
    rng = np.random.default_rng(7)

    def producer():  # a burst of 6, then Poisson arrivals with a mean gap of 3 ms
        for k, (si, p, pi) in enumerate(jobs):
            tickets[k] = srv.submit(gs[si], p, pi, camera=scenes[si].camera_for(p.width, p.height))
            if k >= 5:
                time.sleep(float(rng.exponential(0.003)))

    th = threading.Thread(target=producer)
    th.start()
    th.join()
    results = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    overlapped = 0
    for k, ((si, p, pi), (film, times)) in enumerate(zip(jobs, results)):
        _same(film, _alone(gpu_ctx, scenes[si], p, pi))
        assert times["submitted"] <= times["admitted"] <= times["finished"]
        overlapped += any(o["admitted"] < times["finished"] and times["admitted"] < o["finished"]
                          for j, (_, o) in enumerate(results) if j != k)
    assert st["jobs_done"] == len(jobs) and st["jobs_failed"] == 0
    assert st["samples_done"] == sum(r[1]["samples"] for r in results)
    spans = [(round(r[1]["submitted"], 4), round(r[1]["admitted"], 4), round(r[1]["finished"], 4))
             for r in results]
    assert overlapped > 0, (spans, st)  # jobs shared the device


def test_admission_keeps_films_within_the_budget(gpu_ctx):
    sc = S.cornell_room(48, 48)
    g = gpu_ctx.scene(sc)
    p = S.cornell_params(48, 48, spp_side=2)
    probe = Server(gpu_ctx, slots=4096)
    base = probe.stats()["bytes_in_use"]
    probe.close()
    film_bytes = 48 * 48 * 16
    srv = Server(gpu_ctx, slots=4096, hbm_budget_bytes=base + film_bytes + film_bytes // 2)
    tickets = [srv.submit(g, p, k) for k in range(5)]
    res = [srv.wait(t) for t in tickets]
    st = srv.stats()
    with pytest.raises(BlingError) as e:  # a film larger than the whole budget
        srv.submit(g, S.cornell_params(96, 96, spp_side=1), 0)
    assert e.value.code == abi.BLING_ERR_BOUNDS
    srv.close()
    assert st["peak_bytes_in_use"] <= base + film_bytes + film_bytes // 2
    for a, b in zip(res, res[1:]):  # one film at a time: each admitted after the previous finished
        assert b[1]["admitted"] >= a[1]["finished"]
    ref = _alone(gpu_ctx, sc, p, 3)
    _same(res[3][0], ref)


def test_wait_timeout_and_errors(gpu_ctx):
    sc = S.heightfield_scene(ns=257, n_spheres=64, width=64, height=64, env_size=(64, 32))
    g = gpu_ctx.scene(sc)
    srv = Server(gpu_ctx, slots=4096, iters_per_step=1)
    t = srv.submit(g, S.heightfield_params(64, 64, spp_side=8, max_depth=8), 0)
    with pytest.raises(BlingError) as e:
        srv.wait(t, timeout_ms=0)
    assert e.value.code == abi.BLING_ERR_TIMEOUT
    film, times = srv.wait(t)
    assert film[..., 0].sum() > 0 and times["finished"] >= times["admitted"]
    with pytest.raises(BlingError):
        srv.wait(t)  # the ticket is forgotten once waited for
    bad = S.heightfield_params(64, 64, spp_side=8)
    bad.strata_x = 0
    with pytest.raises(BlingError):
        srv.submit(g, bad, 0)
    srv.close()


def test_submit_does_not_wait_for_the_running_step(gpu_ctx):
    """A job submitted while a long step runs on the device is queued at
    once: submission takes no lock that the worker holds during a step."""
    sc = S.heightfield_scene(ns=257, n_spheres=64, width=256, height=256, env_size=(64, 32))
    g = gpu_ctx.scene(sc)
    srv = Server(gpu_ctx, slots=1 << 20, iters_per_step=64)
    # 17M path samples: far longer than the submissions below
    big = srv.submit(g, S.heightfield_params(256, 256, spp_side=16, max_depth=8), 0)
    time.sleep(0.02)  # the worker is inside a step by now
    small = S.heightfield_params(256, 256, spp_side=1, max_depth=3)
    t0 = time.perf_counter()
    tickets = [srv.submit(g, small, k) for k in range(8)]
    dt = time.perf_counter() - t0
    res_big = srv.wait(big)
    res = [srv.wait(t) for t in tickets]
    srv.close()
    assert dt < 0.02, dt
    assert all(r[1]["submitted"] < res_big[1]["finished"] for r in res)


def test_short_job_overtakes_a_long_one():
    """Samples go to the wavefront in slices, shortest remaining job first:
    a short job submitted while a long one runs finishes long before it, and
    both films are the ones their jobs render alone."""
    from bling_gb300.api import Context
    ctx = Context(device=0)
    try:
        sc = S.heightfield_scene(ns=257, n_spheres=64, width=512, height=512, env_size=(64, 32))
        g = ctx.scene(sc)
        srv = Server(ctx, slots=1 << 20, iters_per_step=8)
        long_p = S.heightfield_params(512, 512, spp_side=16, max_depth=8)  # 67M samples
        short_p = S.heightfield_params(96, 96, spp_side=2, max_depth=4)
        t_long = srv.submit(g, long_p, 0, camera=sc.camera_for(512, 512))
        time.sleep(0.01)
        t_short = srv.submit(g, short_p, 1, camera=sc.camera_for(96, 96))
        f_short, times_short = srv.wait(t_short)
        f_long, times_long = srv.wait(t_long)
        srv.close()
        assert times_short["finished"] < times_long["finished"]
        assert (times_short["finished"] - times_short["submitted"]) < \
            0.5 * (times_long["finished"] - times_long["submitted"])
        _same(f_short, _alone(ctx, sc, short_p, 1))
        _same(f_long, _alone(ctx, sc, long_p, 0))
    finally:
        ctx.close()


def test_failed_step_drops_the_running_jobs_and_later_jobs_render_as_alone(gpu_ctx):
    """A step that fails (injected on the host after one good step, so paths
    of the running job are in flight) fails the running job; the batch drops
    that job's work before its film is released, and a job submitted
    afterwards -- whose film may reuse the released memory -- renders exactly
    as it does alone."""
    sc = S.cornell_room(64, 64)
    g = gpu_ctx.scene(sc)
    srv = Server(gpu_ctx, slots=8192, iters_per_step=2)
    srv.debug_fail_step(1)
    p_first = S.cornell_params(64, 64, spp_side=4, max_depth=5, rr_depth=3, seed=11)
    t = srv.submit(g, p_first, 0)
    with pytest.raises(BlingError) as e:
        srv.wait(t)
    assert e.value.code == abi.BLING_ERR_CUDA
    assert "injected" in str(e.value)
    p_next = S.cornell_params(64, 64, spp_side=2, max_depth=5, rr_depth=3, seed=12)
    tickets = [srv.submit(g, p_next, k) for k in range(2)]
    res = [srv.wait(tk) for tk in tickets]
    st = srv.stats()
    srv.close()
    assert st["jobs_failed"] == 1 and st["jobs_done"] == 2
    for k, (film, _) in enumerate(res):
        _same(film, _alone(gpu_ctx, sc, p_next, k))
