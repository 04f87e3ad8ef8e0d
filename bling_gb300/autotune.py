"""Autotuner for the batched wavefront (``bling_batch``).

Picks the block size, the queue capacity (path slots), the BVH leaf size,
whether to bin rays by Morton order, and the graph mode for a batch of jobs,
by timing short trial runs on the GPU:

* the trial workload is the batch itself at reduced sample counts: every job
  keeps its scene, image size and depth, with one sample per pixel
  (``trial_strata``), so the trial sees the real mix of scenes and path
  lengths in a fraction of the time;
* leaf sizes other than the scenes' own are tried by rebuilding the scenes of
  the trial (``scene_factory``), on a fresh context per leaf size;
* each configuration runs a warm-up batch and then a timed one; the score is
  path samples per second over the timed batch.

Results are cached per device name and workload signature in a JSON file
when ``cache`` is given.  Nothing here changes what a job renders: every
configuration gives each job the same film up to the order of float
additions (tests/test_batch_gpu.py checks this for every option).
"""
from __future__ import annotations

import hashlib
import itertools
import json
import math
import time
from dataclasses import asdict, dataclass
from pathlib import Path

from . import abi
from .api import Batch, Context


@dataclass(frozen=True)
class BatchConfig:
    block_size: int = 128
    slots: int = 1 << 21
    sort_rays: bool = False
    graph_mode: int = abi.BATCH_GRAPH
    leaf_size: int = 4

    def batch_kwargs(self) -> dict:
        return {"block_size": self.block_size, "slots": self.slots, "sort_rays": self.sort_rays,
                "graph_mode": self.graph_mode, "iters_per_launch": 16}


DEFAULT_GRID = {
    "block_size": (64, 128),
    "slots": (1 << 20, 1 << 21, 1 << 22),
    "sort_rays": (False, True),
    "graph_mode": (abi.BATCH_GRAPH, abi.BATCH_DEVICE_LOOP),
    "leaf_size": (2, 4, 8),
}


def _trial_params(p, strata):
    q = abi.RenderParams()
    C_fields = [f for f, _ in abi.RenderParams._fields_]
    for f in C_fields:
        setattr(q, f, getattr(p, f))
    q.strata_x, q.strata_y = strata
    return q


def _signature(jobs, device_name) -> str:
    h = hashlib.sha256(device_name.encode())
    for scene_key, p in jobs:
        h.update(repr((scene_key, p.width, p.height, p.strata_x, p.strata_y, p.max_depth,
                       p.rr_depth)).encode())
    return h.hexdigest()[:16]


def extent_samples(p) -> int:
    """path samples of one pass: the filter-padded sample extent
    (imageWindow', Image.hs:170-176) times the strata"""
    if p.filter_kind == abi.FILTER_BOX:
        fw = fh = 0.5
    else:
        fw, fh = p.filter_params[0], p.filter_params[1]
    nx = math.floor(0.5 + p.width + fw) - math.floor(0.5 - fw) + 1
    ny = math.floor(0.5 + p.height + fh) - math.floor(0.5 - fh) + 1
    return nx * ny * p.strata_x * p.strata_y


def _time_batch(ctx, jobs, cfg: BatchConfig, films) -> float:
    """path samples per second of one batch of the jobs (after a warm-up batch
    of the first job, which captures the graphs)"""
    b = Batch(ctx, **cfg.batch_kwargs())
    try:
        g, p = jobs[0]
        b.submit(g, films[0], p, 0)
        b.run()
        for f in films:
            f.clear()
        t0 = time.perf_counter()
        for (g, p), f in zip(jobs, films):
            b.submit(g, f, p, 1)
        b.run()
        dt = time.perf_counter() - t0
        return sum(extent_samples(p) for _, p in jobs) / dt
    finally:
        b.close()


def autotune(scenes, params, scene_factory=None, grid=None, trial_strata=(1, 1), max_trials=None,
             cache: str | Path | None = None, device: int = 0, log=None) -> tuple[BatchConfig, list]:
    """Returns (best configuration, [(config, samples/s), ...]).

    scenes: host ``Scene`` objects (or GpuScenes when ``scene_factory`` is None
    and only the scenes' own leaf size is tried); params: one
    ``abi.RenderParams`` per job; scene_factory(scene, ctx) -> GpuScene builds
    a scene on a context (whose leaf size the tuner chooses)."""
    grid = dict(DEFAULT_GRID if grid is None else grid)
    if scene_factory is None:
        grid["leaf_size"] = (0,)  # the scenes as given
    trial = [_trial_params(p, trial_strata) for p in params]
    import torch  # device name for the cache key only
    name = torch.cuda.get_device_name(device) if torch.cuda.is_available() else "cpu"
    sig = _signature([(k, p) for k, p in enumerate(trial)], name + json.dumps(grid, default=str))
    if cache is not None and Path(cache).exists():
        data = json.loads(Path(cache).read_text())
        if sig in data:
            return BatchConfig(**data[sig]["best"]), [(BatchConfig(**c), s) for c, s in
                                                      data[sig]["results"]]
    results = []
    keys = ("block_size", "slots", "sort_rays", "graph_mode")
    for leaf in grid["leaf_size"]:
        ctx = Context(device=device, bvh_leaf_size=leaf) if scene_factory else None
        try:
            if scene_factory:
                gs = [scene_factory(s, ctx) for s in scenes]
                use_ctx = ctx
            else:
                gs = list(scenes)
                use_ctx = gs[0].ctx
            jobs = list(zip(gs, trial))
            films = [use_ctx.film(p.width, p.height) for p in trial]
            combos = list(itertools.product(*(grid[k] for k in keys)))
            for vals in combos:
                cfg = BatchConfig(**dict(zip(keys, vals)), leaf_size=leaf)
                if max_trials is not None and len(results) >= max_trials:
                    break
                rate = _time_batch(use_ctx, jobs, cfg, films)
                results.append((cfg, rate))
                if log:
                    log(f"{cfg} -> {rate / 1e6:.1f} M samples/s")
            for f in films:
                f.close()
        finally:
            if ctx is not None:
                ctx.close()
    best = max(results, key=lambda r: r[1])[0]
    if cache is not None:
        p = Path(cache)
        data = json.loads(p.read_text()) if p.exists() else {}
        data[sig] = {"best": asdict(best), "results": [(asdict(c), s) for c, s in results]}
        p.write_text(json.dumps(data, indent=1))
    return best, results
