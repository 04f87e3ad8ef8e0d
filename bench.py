"""Benchmark of the GB300 path-tracing core.

Workload (one "step"): the ray-cast microbenchmark -- a 1M-triangle soup
(uniform-random triangles in [-1,1]^3, edge lengths ~U(0.005, 0.05), FP32
vertices, int32 indices) queried by 16M closest-hit rays (origins on a sphere
of radius 3, directions towards random points of the unit ball, tmax = inf)
and by an 8M any-hit subset (tmax = distance to a second random point).
Metric: Mrays/s over all traversal queries (closest + any).

  value   device-resident throughput: rays already in HBM, CUDA events on the
          launching stream, L2 flushed between steps (the 512 MB ray buffer is
          also larger than L2; the BVH stays resident like any scene)
  e2e     the same rays through the C-ABI host-buffer calls
          (bling_trace_closest / bling_trace_any) from pinned memory: H2D copy
          of the rays and D2H copy of (t, prim) / hit flags inside the timed
          region
  cpu_baseline / --impl reference
          the reference's algorithm on the host cores: the CPU oracle's
          restatement of its kd-tree (exact-event SAH build and front-to-back
          traversal, Primitive/KdTree.hs) and intersection code, on a bounded
          sample of the same rays, all host cores (the Haskell reference has
          no toolchain here); kd-tree build time and node/leaf counts beside
          it

Multi-GPU: the path does not shard -- `--gpus N` runs N independent replicas
(one per rank, torchrun), `value` = all ranks' rays / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_TRIS = 1 << 20
N_RAYS = 1 << 24
N_ANY = N_RAYS // 2
CPU_SAMPLE_RAYS = 1 << 20


def l2_read_peak(device: int):
    """L2 read bandwidth measured on this GPU by the project's probe kernel
    (libbling_probe.so: 16-byte ld.global.cg over a 64 MB working set that
    stays in L2, 20 repeats, 2 blocks of 512 threads per SM); best of 3."""
    import ctypes as C
    lib = ROOT / "bling_gb300" / "libbling_probe.so"
    if not lib.exists():
        return None
    L = C.CDLL(str(lib))
    L.bling_probe_l2_read_gbs.restype = C.c_double
    L.bling_probe_l2_read_gbs.argtypes = [C.c_int, C.c_size_t, C.c_int, C.c_int,
                                          C.POINTER(C.c_float), C.POINTER(C.c_size_t)]
    best, ms, ws = -1.0, C.c_float(), C.c_size_t()
    for _ in range(3):
        best = max(best, L.bling_probe_l2_read_gbs(device, 64 << 20, 20, 2, C.byref(ms),
                                                   C.byref(ws)))
    if best <= 0:
        return None
    return {"gbs": round(best, 1), "working_set_bytes": ws.value, "repeats": 20,
            "how": "ld.global.cg.v4 over a 64 MB L2-resident working set, best of 3"}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.dev), "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x: float, world: int, device=None) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def kd_oracle(scene):
    """The CPU oracle of a scene with the reference's kd-tree built: returns
    (oracle, {"build_s", kd-tree statistics})."""
    from oracle.oracle import OracleScene
    o = OracleScene(scene)
    t0 = time.perf_counter()
    st = o.kdtree()
    info = {"build_s": round(time.perf_counter() - t0, 3)}
    info.update(st)
    o.use_kdtree(True)
    return o, info


def cpu_oracle_rate(soup, rays_np, ra_np, n_sample: int):
    """Mrays/s of the reference's kd-tree traversal on the host cores (closest
    + any over a bounded sample)."""
    o, kd = kd_oracle(soup)
    nc = n_sample
    na = n_sample // 2
    rc = np.ascontiguousarray(rays_np[:, :nc])
    rr = np.ascontiguousarray(ra_np[:, :na])
    t0 = time.perf_counter()
    o.closest_kd(rc)
    o.any_kd(rr)
    dt = time.perf_counter() - t0
    cores = os.cpu_count() or 1
    return ((nc + na) / dt / 1e6, cores, dt,
            f"{nc} closest + {na} any-hit rays of the same workload through the kd-tree", kd)


def run_reference(args):
    """--impl reference: the reference's algorithm on the host cores -- the
    CPU oracle's restatement of its kd-tree build and traversal
    (Primitive/KdTree.hs:81-246) and of its intersection code; the Haskell
    reference has no toolchain here."""
    world, rank, _ = dist_env()
    if world > 1 and rank != 0:
        return
    from bling_gb300 import scene as S
    from oracle import build as ob
    ob.build()
    soup = S.triangle_soup(N_TRIS, seed=1)
    rays = S.soup_rays(N_RAYS if args.full_rays else (args.cpu_rays * 2), seed=2)
    ra = S.soup_rays(N_RAYS if args.full_rays else (args.cpu_rays * 2), seed=3, any_hit=True)
    o, kd = kd_oracle(soup)
    n = args.cpu_rays
    rc = np.ascontiguousarray(rays[:, :n])
    rr = np.ascontiguousarray(ra[:, :n // 2])
    for _ in range(args.warmup):
        o.closest_kd(rc[:, : max(1, n // 16)])
    times = []
    visits = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, _, _, cc = o.closest_kd(rc)
        _, ca = o.any_kd(rr)
        times.append(time.perf_counter() - t0)
        visits = {"closest_nodes_per_ray": round(cc["nodes"] / n, 2),
                  "closest_prims_per_ray": round(cc["prims"] / n, 2),
                  "any_nodes_per_ray": round(ca["nodes"] / max(1, n // 2), 2),
                  "any_prims_per_ray": round(ca["prims"] / max(1, n // 2), 2)}
    dt = float(np.mean(times))
    val = (n + n // 2) / dt / 1e6
    cores = os.cpu_count() or 1
    line = {
        "impl": "reference", "metric": "Mrays/s", "value": round(val, 3), "unit": "Mrays/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, world),
        "cpu_baseline": {"value": round(val, 3), "unit": "Mrays/s", "cores": cores, "kind": "port",
                         "sample": f"{n} closest + {n // 2} any-hit rays per step (of 16M + 8M) "
                                   "through the kd-tree"},
        "e2e": {"value": round(val, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "kdtree": dict(kd, **(visits or {})),
        "note": "reference is Haskell (GHC absent); its kd-tree and intersection code run as the "
                "C++ oracle restatement (oracle/kdtree.h, oracle/oracle.cpp)",
    }
    print(json.dumps(line), flush=True)


def workload_config(args, world):
    return {"workload": "ray-cast microbench: 1M-tri soup, 16M closest + 8M any-hit rays",
            "triangles": N_TRIS, "rays_closest": N_RAYS, "rays_any": N_ANY,
            "l2": "flushed between steps (256 MB write); ray buffers 768 MB > L2",
            "parallelism": f"replicas x{world}"}


def measure_e2e(ctx, g, rays, ra, flush, args, world, dev):
    """The same rays end to end through the host-buffer C-ABI calls: H2D copy
    of the rays from pinned memory, traversal, D2H copy of (t, prim) and of
    the any-hit flags, all inside the timed region."""
    import ctypes as C

    import torch

    from bling_gb300.api import lib
    h_rays = torch.from_numpy(rays).pin_memory().numpy()
    h_any = torch.from_numpy(ra).pin_memory().numpy()
    h_t = torch.empty(N_RAYS, dtype=torch.float32).pin_memory().numpy()
    h_p = torch.empty(N_RAYS, dtype=torch.int32).pin_memory().numpy()
    h_h = torch.empty(N_ANY, dtype=torch.uint8).pin_memory().numpy()
    L = lib()
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731

    def e2e_step():
        ctx.check(L.bling_trace_closest(g.h, fp(h_rays), N_RAYS, fp(h_t),
                                        h_p.ctypes.data_as(C.POINTER(C.c_int32)),
                                        C.POINTER(C.c_float)()))
        ctx.check(L.bling_trace_any(g.h, fp(h_any), N_ANY, h_h.ctypes.data_as(C.POINTER(C.c_uint8))))

    for _ in range(max(1, args.warmup)):
        e2e_step()
    barrier(world)
    e2e_times = []
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_times.append(time.perf_counter() - t0)
    e2e_total = max_over_ranks(sum(e2e_times), world, dev)
    value = world * (N_RAYS + N_ANY) * args.steps / e2e_total / 1e6
    return {"value": round(value, 2), "unit": "Mrays/s", "h2d_bytes_per_step": N_RAYS * 32 + N_ANY * 32,
            "d2h_bytes_per_step": N_RAYS * 8 + N_ANY * 1}


def _cpu_render_rate(sc, p, bands):
    """path samples/s of the oracle's path integrator through the reference's
    kd-tree, all host threads, over `bands` = [(row_begin, row_end), ...] of
    the sample extent; returns (cpu_baseline dict without "sample", kd info)"""
    o, kd = kd_oracle(sc)
    samples, dt = 0, 0.0
    for rb, re_ in bands:
        t0 = time.perf_counter()
        _, st = o.render_pass(p, 0, rows=(rb, re_))
        dt += time.perf_counter() - t0
        samples += st["path_samples"]
    return {"value": round(samples / dt, 1), "unit": "path samples/s",
            "cores": os.cpu_count() or 1, "kind": "port"}, kd


def _gpu_built_pass(sc, p, stream):
    """BVH build and scene creation times with the tree built on the GPU
    (BLING_FLAG_GPU_BVH), and the time of one pass over that tree"""
    import torch

    from bling_gb300.api import Context
    ctx = Context(device=torch.cuda.current_device(), gpu_bvh=True)
    ctx.set_stream(stream.cuda_stream)
    g = ctx.scene(sc)
    st = g.stats()
    film = ctx.film(p.width, p.height, fp64=True)
    g.render_pass(film, p, 0)  # warm-up
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record(stream)
    g.render_pass(film, p, 1)
    ev[1].record(stream)
    torch.cuda.synchronize()
    out = {"bvh_build_ms": round(st["bvh_build_ms"], 1),
           "scene_create_ms": round(st["scene_build_ms"], 1), "bvh_nodes": st["bvh_nodes"],
           "ms_per_pass": round(ev[0].elapsed_time(ev[1]), 3)}
    ctx.close()
    return out


def measure_render(ctx, stream, args):
    """The path integrator on the two render workloads (secondary lines):
    path samples/s and Mrays/s (camera, continuation, BSDF-MIS and shadow
    queries, counted on the device) per pass, CUDA events on the stream.  The
    large-mesh workload accumulates into an FP64-compensated film, as its
    configuration asks.  Beside each: the oracle's path integrator through the
    reference's kd-tree on the host cores (the whole Cornell image; 8 bands
    of 2 rows spread over the heightfield image)."""
    import torch

    from bling_gb300 import scene as S
    out = {}
    cases = [("cornell_256x256_16spp_depth5", S.cornell_room(256, 256),
              S.cornell_params(256, 256, spp_side=4, max_depth=5, rr_depth=3), 10, False)]
    if not args.no_heightfield:
        cases.append(("heightfield_8.4Mtri_4096spheres_1920x1080_64spp_depth8",
                      S.heightfield_scene(), S.heightfield_params(1920, 1080, spp_side=8), 2, True))
    for name, sc, p, passes, fp64 in cases:
        t0 = time.perf_counter()
        g = ctx.scene(sc)
        build_s = time.perf_counter() - t0
        film = ctx.film(p.width, p.height, fp64=fp64)
        g.render_pass(film, p, 0)  # warm-up pass
        s0 = g.stats()
        times = []
        for k in range(passes):
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            ev[0].record(stream)
            g.render_pass(film, p, k + 1)
            ev[1].record(stream)
            torch.cuda.synchronize()
            times.append(ev[0].elapsed_time(ev[1]) / 1e3)
        s1 = g.stats()
        tot = sum(times)
        rays = (s1["rays_closest"] - s0["rays_closest"]) + (s1["rays_any"] - s0["rays_any"])
        out[name] = {
            "path_samples_per_s": round((s1["path_samples"] - s0["path_samples"]) / tot, 1),
            "mrays_per_s": round(rays / tot / 1e6, 2),
            "ms_per_pass": round(tot / passes * 1e3, 3), "passes": passes,
            "rays_per_path": round(rays / max(1, s1["path_samples"] - s0["path_samples"]), 3),
            "scene_build_s": round(build_s, 3), "bvh_build_ms": round(s1["bvh_build_ms"], 1),
            "scene_create_ms": round(s1["scene_build_ms"], 1),
            "nonfinite_drops": s1["nonfinite_drops"],
            "film": "fp64-compensated" if fp64 else "fp32"}
        if s1["nonfinite_pass"] >= 0:  # the latest pass's first dropped sample
            out[name]["nonfinite_first"] = {"pass": s1["nonfinite_pass"],
                                            "pixel": list(s1["nonfinite_pixel"]),
                                            "sample": s1["nonfinite_sample"]}
        if fp64:  # the large mesh: the same pass over a BVH built on the GPU
            out[name]["gpu_built_bvh"] = _gpu_built_pass(sc, p, stream)
        if not args.no_cpu_baseline:
            ny = p.height + 2  # box filter: the sample extent is one pixel wider on each side
            if name.startswith("cornell"):
                bands, what = [(0, ny)], f"the whole {p.width + 2} x {ny} sample extent"
            else:
                bands = [(int(k * ny / 8) + ny // 16, int(k * ny / 8) + ny // 16 + 2)
                         for k in range(8)]
                what = (f"8 bands of 2 rows spread over the {p.width + 2} x {ny} sample extent "
                        f"(rows {', '.join(str(b[0]) for b in bands)})")
            cpu, kd = _cpu_render_rate(sc, p, bands)
            cpu["sample"] = f"{what}, {p.strata_x * p.strata_y} spp, one pass, kd-tree"
            out[name]["cpu_baseline"] = cpu
            out[name]["cpu_kdtree"] = kd
        del g, film
    return out


def measure_light(ctx, stream, args):
    """The light tracer on the Cornell room (secondary line): photons/s and
    Mrays/s (emission, continuation and camera-connection queries, counted on
    the device) per pass of `--light-photons` photons, CUDA events on the
    stream; the oracle's light tracer on a bounded photon sample beside it."""
    import torch

    from bling_gb300 import scene as S
    W = H = 256
    n = args.light_photons
    sc = S.cornell_room(W, H)
    g = ctx.scene(sc)
    film = ctx.film(W, H)
    g.light_pass(film, n, seed=1, pass_index=0)  # warm-up pass
    s0 = g.stats()
    times = []
    passes = 3
    for k in range(passes):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record(stream)
        g.light_pass(film, n, seed=1, pass_index=k + 1)
        ev[1].record(stream)
        torch.cuda.synchronize()
        times.append(ev[0].elapsed_time(ev[1]) / 1e3)
    s1 = g.stats()
    tot = sum(times)
    rays = (s1["rays_closest"] - s0["rays_closest"]) + (s1["rays_any"] - s0["rays_any"])
    out = {"workload": f"cornell_{W}x{H}_{n}_photons_per_pass",
           "photons_per_s": round(passes * n / tot, 1), "mrays_per_s": round(rays / tot / 1e6, 2),
           "ms_per_pass": round(tot / passes * 1e3, 3), "passes": passes,
           "rays_per_photon": round(rays / (passes * n), 3),
           "splats_per_photon": round((s1["light_splats"] - s0["light_splats"]) / (passes * n), 3),
           "nonfinite_drops": s1["nonfinite_drops"]}
    if not args.no_cpu_baseline:
        o, _ = kd_oracle(sc)
        m = 400_000
        t0 = time.perf_counter()
        o.light_pass(W, H, m, seed=1, pass_index=1)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(m / dt, 1), "unit": "photons/s",
                               "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": f"{m} photons of one pass, all host threads, kd-tree"}
    del g, film
    return out


def measure_sppm(ctx, stream, args):
    """SPPM on the Cornell room (secondary line): one pass = a camera pass
    (one sample per pixel, specular trees to depth 5), the hit-point hash and
    `--sppm-photons` photons; passes/s, photons/s and Mrays/s, CUDA events on
    the stream; the oracle on one bounded pass beside it."""
    import torch

    from bling_gb300 import abi
    from bling_gb300 import scene as S
    W = H = 256
    n = args.sppm_photons
    sc = S.cornell_room(W, H)
    sp = abi.sppm_params(n, max_depth=5, radius=0.01, alpha=0.7, seed=1)
    g = ctx.scene(sc)
    film = ctx.film(W, H)
    g.sppm_pass(film, sp, 0)  # warm-up pass
    s0 = g.stats()
    times = []
    passes = 3
    for k in range(passes):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record(stream)
        g.sppm_pass(film, sp, k + 1)
        ev[1].record(stream)
        torch.cuda.synchronize()
        times.append(ev[0].elapsed_time(ev[1]) / 1e3)
    s1 = g.stats()
    tot = sum(times)
    sn = int(np.ceil(np.sqrt(np.float32(n))))
    rays = s1["rays_closest"] - s0["rays_closest"]
    out = {"workload": f"cornell_{W}x{H}_{sn * sn}_photons_depth5_r0.01",
           "passes_per_s": round(passes / tot, 2), "ms_per_pass": round(tot / passes * 1e3, 3),
           "photons_per_s": round(passes * sn * sn / tot, 1), "mrays_per_s": round(rays / tot / 1e6, 2),
           "splats_per_photon": round((s1["light_splats"] - s0["light_splats"]) / (passes * sn * sn), 3),
           "passes": passes, "nonfinite_drops": s1["nonfinite_drops"]}
    if not args.no_cpu_baseline:
        o, _ = kd_oracle(sc)
        m = 250_000
        spc = abi.sppm_params(m, max_depth=5, radius=0.01, alpha=0.7, seed=1)
        t0 = time.perf_counter()
        o.sppm_pass(spc, W, H, 0)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(m / dt, 1), "unit": "photons/s",
                               "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": f"one pass with {m} photons (camera pass included), "
                                         "all host threads, kd-tree"}
    del g, film
    return out


def run_sppm_profile(args):
    """Only SPPM passes of the Cornell room (for an ncu launch list)."""
    from bling_gb300 import abi
    from bling_gb300 import scene as S
    from bling_gb300.api import Context
    ctx = Context(device=0)
    g = ctx.scene(S.cornell_room(256, 256))
    film = ctx.film(256, 256)
    sp = abi.sppm_params(args.sppm_photons, max_depth=5, radius=0.01, alpha=0.7, seed=1)
    for k in range(args.warmup + args.steps):
        g.sppm_pass(film, sp, k)
    st = g.stats()
    print(json.dumps({"sppm_profile": True, "photons": args.sppm_photons,
                      "passes": args.warmup + args.steps, "rays_closest": st["rays_closest"],
                      "splats": st["light_splats"]}))


def run_light_profile(args):
    """Only light passes of the Cornell room (for an ncu launch list)."""
    from bling_gb300.api import Context
    from bling_gb300 import scene as S
    ctx = Context(device=0)
    g = ctx.scene(S.cornell_room(256, 256))
    film = ctx.film(256, 256)
    for k in range(args.warmup + args.steps):
        g.light_pass(film, args.light_photons, seed=1, pass_index=k)
    st = g.stats()
    print(json.dumps({"light_profile": True, "photons": args.light_photons,
                      "passes": args.warmup + args.steps, "rays_closest": st["rays_closest"],
                      "rays_any": st["rays_any"], "splats": st["light_splats"]}))


def _extent_samples(p):
    from bling_gb300.autotune import extent_samples
    return extent_samples(p)


def _films_equal(a, b, spp=1):
    """equal samples up to the order of float additions (box-filter weights
    exact): a sum of n binary32 terms in another order differs by at most
    about n * 2^-24 of the sum of their magnitudes, so the relative bar grows
    with the samples per pixel (at least 1e-5)"""
    return _film_diff(a, b, spp)["equal"]


def _film_diff(a, b, spp=1):
    if not np.array_equal(a[..., 0], b[..., 0]):
        return {"equal": False, "weights_differ": True}
    rtol = max(1e-5, 2.0 * spp * 2.0 ** -24)
    scale = float(np.abs(b[..., 1:]).max()) + 1e-30
    err = np.abs(a[..., 1:] - b[..., 1:])
    ok = err <= 1e-6 * scale + rtol * np.abs(b[..., 1:])
    rel = float((err / (np.abs(b[..., 1:]) + 1e-6 * scale)).max())
    return {"equal": bool(ok.all()), "rtol": rtol, "max_rel_err": rel,
            "values_off": int((~ok).sum())}


def measure_batched(args):
    """The batched workload: `--batch-instances` scene instances (seeded soup
    plus spheres, triangle counts log-uniform in [10k, 2M], square images with
    sides uniform in [128, 1024], 4-256 spp, max depth 3-10), one pass each.
    Plain: one bling_render_pass per job, back to back.  Batched: one batch
    of all jobs (path regeneration, a CUDA graph per iteration) in the
    configuration the autotuner picks on a trial at 1 spp.  Both sides trace
    the same samples with the same random numbers, so the images, and their
    RMSE against any reference, are equal up to the order of float additions;
    `equal_images` reports the check."""
    import torch

    from bling_gb300 import autotune
    from bling_gb300 import scene as S
    from bling_gb300.api import Batch, Context
    t0 = time.perf_counter()
    inst = S.batch_instances(n=args.batch_instances)
    gen_s = time.perf_counter() - t0
    params = [i.params for i in inst]
    samples = sum(_extent_samples(p) for p in params)
    # autotune on a quarter of the instances (leaf sizes rebuild those scenes)
    sub = inst[:: max(1, len(inst) // 16)][:16]
    t0 = time.perf_counter()
    best, trials = autotune.autotune([i.scene for i in sub], [i.params for i in sub],
                                     scene_factory=lambda sc, c: c.scene(sc))
    tune_s = time.perf_counter() - t0
    ctx = Context(device=0, bvh_leaf_size=best.leaf_size)
    t0 = time.perf_counter()
    gs = [ctx.scene(i.scene) for i in inst]
    build_s = time.perf_counter() - t0
    films = [ctx.film(p.width, p.height) for p in params]
    gs[0].render_pass(films[0], params[0], 0)  # warm-up
    films[0].clear()
    st0 = [g.stats() for g in gs]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for g, p, f in zip(gs, params, films):
        g.render_pass(f, p, 1)
    plain_s = time.perf_counter() - t0
    st1 = [g.stats() for g in gs]
    rays = sum((b["rays_closest"] - a["rays_closest"]) + (b["rays_any"] - a["rays_any"])
               for a, b in zip(st0, st1))
    ref = [f.read() for f in films]
    b = Batch(ctx, **best.batch_kwargs())
    b.submit(gs[0], films[0], params[0], 0)  # warm-up (graph capture)
    b.run()
    for f in films:
        f.clear()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for g, p, f in zip(gs, params, films):
        b.submit(g, f, p, 1)
    b.run()
    batch_s = time.perf_counter() - t0
    bst = b.stats()
    equal = all(_films_equal(f.read(), r, p.strata_x * p.strata_y)
                for f, r, p in zip(films, ref, params))
    b.close()
    out = {
        "instances": len(inst), "triangles": sum(i.n_tris for i in inst),
        "path_samples": samples, "scene_gen_s": round(gen_s, 2), "bvh_build_s": round(build_s, 2),
        "plain_per_job": {"s": round(plain_s, 3), "path_samples_per_s": round(samples / plain_s, 1),
                          "mrays_per_s": round(rays / plain_s / 1e6, 2)},
        "batched": {"s": round(batch_s, 3), "path_samples_per_s": round(samples / batch_s, 1),
                    "mrays_per_s": round((bst["rays_closest"] + bst["rays_any"]) / batch_s / 1e6, 2),
                    "iterations": bst["iterations"]},
        "speedup": round(plain_s / batch_s, 3), "equal_images": equal,
        "autotuned": {**best.__dict__, "trials": len(trials), "tune_s": round(tune_s, 1),
                      "trial": "1 spp, every 4th instance, leaf sizes 2/4/8"},
    }
    ctx.close()
    return out


def _pct(xs, q):
    return float(np.percentile(np.asarray(xs), q)) if xs else None


def measure_serving(args):
    """The serving workload: eight resident scenes (6M triangles), jobs
    arriving as a Poisson process at 200/s, each on one scene at a square
    size log-uniform in [128, 1024] and 16-512 spp (log-uniform), admitted
    under a 40 GiB budget and merged into one wavefront by the render server.
    Reported: p50/p99 latency (arrival to film on the host) and path
    samples/s over the run, next to the same jobs run alone one after the
    other through bling_render_pass (latency of that FIFO from the same
    arrivals, each job's service time measured).

    A second line, `small_jobs`, runs the same comparison for preview-sized
    traffic on the same scenes: 256 jobs at 2000/s, sides log-uniform in
    [64, 128], 1-16 spp."""
    from bling_gb300 import scene as S
    from bling_gb300.api import Context
    ctx = Context(device=0)
    t0 = time.perf_counter()
    scenes = S.serving_scenes()
    gs = [ctx.scene(s) for s in scenes]
    build_s = time.perf_counter() - t0
    out = _serve(args, ctx, scenes, gs, S.serving_jobs(n=args.serving_jobs), 200)
    out["scene_build_s"] = round(build_s, 2)
    out["small_jobs"] = _serve(args, ctx, scenes, gs,
                               S.serving_jobs(n=256, rate=2000.0, seed=43, side_range=(64, 128),
                                              spp_range=(1, 16)), 2000)
    ctx.close()
    return out


def _serve(args, ctx, scenes, gs, jobs, rate):
    import threading

    import torch

    from bling_gb300 import scene as S
    from bling_gb300.api import Server
    cams = [scenes[j.scene].camera_for(j.params.width, j.params.height) for j in jobs]
    samples = [_extent_samples(j.params) for j in jobs]
    # plain: each job alone, in arrival order
    warm = ctx.film(64, 64)
    gs[0].render_pass(warm, S.render_params(64, 64, (1, 1)), 0, camera=scenes[0].camera_for(64, 64))
    service, refs = [], []
    for j, cam in zip(jobs, cams):
        f = ctx.film(j.params.width, j.params.height)
        torch.cuda.synchronize()
        t = time.perf_counter()
        gs[j.scene].render_pass(f, j.params, j.pass_index, camera=cam)
        service.append(time.perf_counter() - t)
        refs.append(f.read())
        f.close()
    plain_lat, free_at = [], 0.0
    for j, s in zip(jobs, service):
        start = max(j.arrival, free_at)
        free_at = start + s
        plain_lat.append(free_at - j.arrival)
    # served: arrivals replayed in real time from a producer thread
    srv = Server(ctx, hbm_budget_bytes=40 << 30, iters_per_step=args.serving_iters)
    w = srv.submit(gs[0], S.render_params(64, 64, (1, 1)), 0, camera=scenes[0].camera_for(64, 64))
    srv.wait(w)  # warm-up (graph capture)
    tickets = [None] * len(jobs)

    def producer():
        t_start = time.perf_counter()
        for k, (j, cam) in enumerate(zip(jobs, cams)):
            d = t_start + j.arrival - time.perf_counter()
            if d > 0:
                time.sleep(d)
            tickets[k] = srv.submit(gs[j.scene], j.params, j.pass_index, camera=cam)

    th = threading.Thread(target=producer)
    th.start()
    th.join()
    res = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    first = min(r[1]["submitted"] for r in res)
    last = max(r[1]["finished"] for r in res)
    lat = [r[1]["finished"] - r[1]["submitted"] for r in res]
    diffs = [_film_diff(r[0], ref, j.params.strata_x * j.params.strata_y)
             for r, ref, j in zip(res, refs, jobs)]
    equal = all(d["equal"] for d in diffs)
    worst = max(range(len(diffs)), key=lambda k: diffs[k].get("max_rel_err", float("inf")))
    tot = sum(samples)
    plain_span = max(j.arrival for j in jobs) + 0.0
    plain_make = max(plain_lat[k] + jobs[k].arrival for k in range(len(jobs)))
    return {
        "scenes": len(scenes), "triangles": sum(s.n_triangles for s in scenes) +
        sum(len(s.shapes) for s in scenes),
        "jobs": len(jobs), "arrival_rate_per_s": rate, "arrivals_span_s": round(plain_span, 3),
        "path_samples": tot,
        "served": {"p50_latency_s": round(_pct(lat, 50), 4), "p99_latency_s": round(_pct(lat, 99), 4),
                   "makespan_s": round(last - first, 3),
                   "path_samples_per_s": round(tot / (last - first), 1),
                   "peak_bytes_in_use": st["peak_bytes_in_use"], "iterations": st["iterations"],
                   "iters_per_step": args.serving_iters},
        "plain_per_job": {"p50_latency_s": round(_pct(plain_lat, 50), 4),
                          "p99_latency_s": round(_pct(plain_lat, 99), 4),
                          "makespan_s": round(plain_make, 3),
                          "path_samples_per_s": round(tot / sum(service), 1)},
        "speedup": round((tot / (last - first)) / (tot / sum(service)), 3),
        "equal_images": equal,
        "largest_film_difference": {"job": worst, **diffs[worst]},
    }


def run_render_profile(args):
    """A small render of the large-mesh workload for profiling (full
    geometry, reduced image): one warm-up pass and `--steps` timed passes."""
    import torch

    from bling_gb300 import build as gb
    gb.build()
    from bling_gb300 import scene as S
    from bling_gb300.api import Context
    w, h, side = args.render_size
    ctx = Context(device=0, bin_rays=args.bin_rays, compact_bvh=args.compact_bvh,
                  gpu_bvh=args.gpu_bvh)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    g = ctx.scene(S.heightfield_scene(width=w, height=h))
    p = S.heightfield_params(w, h, spp_side=side)
    film = ctx.film(w, h)
    g.render_pass(film, p, 0)
    s0 = g.stats()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        g.render_pass(film, p, k + 1)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    s1 = g.stats()
    print(json.dumps({"workload": f"heightfield {w}x{h} {side * side}spp", "passes": args.steps,
                      "bin_rays": args.bin_rays, "gpu_bvh": args.gpu_bvh,
                      "ms_per_pass": dt / args.steps * 1e3,
                      "path_samples_per_s": (s1["path_samples"] - s0["path_samples"]) / dt,
                      "rays_closest": s1["rays_closest"] - s0["rays_closest"],
                      "rays_any": s1["rays_any"] - s0["rays_any"]}), flush=True)


def run_ours(args):
    import torch
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from bling_gb300 import build as gb
    gb.build()
    from bling_gb300 import scene as S
    from bling_gb300.api import Context

    ctx = Context(device=local, wide_bvh=args.wide_bvh, compact_bvh=args.compact_bvh,
                  gpu_bvh=args.gpu_bvh)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    soup = S.triangle_soup(N_TRIS, seed=1)
    rays = S.soup_rays(N_RAYS, seed=2)
    ra = S.soup_rays(N_RAYS, seed=3, any_hit=True)
    ra = np.ascontiguousarray(ra[:, :N_ANY])
    g = ctx.scene(soup)
    st = g.stats()

    d_rays = torch.from_numpy(rays).to(dev)
    d_any = torch.from_numpy(ra).to(dev)
    d_t = torch.empty(N_RAYS, dtype=torch.float32, device=dev)
    d_p = torch.empty(N_RAYS, dtype=torch.int32, device=dev)
    d_h = torch.empty(N_ANY, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step():
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record(stream)
        g.closest_device(d_rays, d_t, d_p)
        ev[1].record(stream)
        g.any_device(d_any, d_h)
        ev[2].record(stream)
        return ev

    for _ in range(args.warmup):
        step()
        flush.fill_(1)
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    step_ms, closest_ms, any_ms = [], [], []
    with ClockSampler(local) as clk:
        time.sleep(0.3)  # let the sampler start before the timed steps
        for _ in range(args.steps):
            flush.fill_(1)
            ev = step()
            torch.cuda.synchronize()
            closest_ms.append(ev[0].elapsed_time(ev[1]))
            any_ms.append(ev[1].elapsed_time(ev[2]))
            step_ms.append(ev[0].elapsed_time(ev[2]))
    torch.cuda.synchronize()
    barrier(world)
    total_s = sum(step_ms) / 1e3
    total_s = max_over_ranks(total_s, world, dev)
    rays_per_step = N_RAYS + N_ANY
    value = world * rays_per_step * args.steps / total_s / 1e6
    hit_frac = float((d_p >= 0).float().mean().item())

    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(ctx, g, rays, ra, flush, args, world, dev)
    render = None
    if not args.no_render and rank == 0:
        render = measure_render(ctx, stream, args)
    light = sppm = None
    if not args.no_light and rank == 0:
        light = measure_light(ctx, stream, args)
    if not args.no_sppm and rank == 0:
        sppm = measure_sppm(ctx, stream, args)
    batched = served = None
    if not args.no_batch and rank == 0:
        batched = measure_batched(args)
    if not args.no_serving and rank == 0:
        served = measure_serving(args)

    # ---- roofline of the dominant kernel (closest hit).  Traversal reads the
    # BVH and the leaf slots out of L2 (the 1M soup's ~100 MB working set
    # stays resident), so the bound is the L2 read bandwidth, measured in this
    # run by the probe kernel.  Algorithmic bytes per ray: 32 (ray) + 8 (t,
    # primitive) + the node bytes of every visit + 48 per leaf slot tested.
    hbm_peak, peak_kind = peaks()
    counts = traversal_counts(g, rays)
    # a visit reads 64 B of a binary node (two child boxes of 32 B each), 80 B
    # of an 8-wide node or 32 B of a compact node (two quantised boxes)
    node_bytes = 80.0 if args.wide_bvh else (32.0 if args.compact_bvh else 64.0)
    box_tests = (8.0 if args.wide_bvh else 2.0) * counts["nodes_per_ray"]
    bytes_per_ray = 32 + 8 + node_bytes * counts["nodes_per_ray"] + 48 * counts["slots_per_ray"]
    closest_s = float(np.mean(closest_ms)) / 1e3
    achieved = bytes_per_ray * N_RAYS / closest_s / 1e9
    prof = profile_traffic()
    l2 = l2_read_peak(local)
    if l2:
        roof = {"bound": "l2", "achieved": round(achieved, 1), "peak": l2["gbs"], "unit": "GB/s",
                "frac": round(achieved / l2["gbs"], 4),
                "peak_source": "measured in this run: " + l2["how"]}
    else:
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                "frac": round(achieved / hbm_peak, 4), "peak_source": peak_kind}
    roof.update({
        "traffic": prof.get("dram_bytes_per_launch") if prof else None,
        "traffic_source": (prof.get("captured") if prof else None),
        "kernel": "k_trace_closest",
        "bvh_layout": ("wide8" if args.wide_bvh else "compact32" if args.compact_bvh
                       else "binary-gpu-built" if args.gpu_bvh else "binary"),
        "algorithmic_bytes_per_ray": round(bytes_per_ray, 1),
        "bytes_per_ray_formula": "32 ray + 8 result + node bytes x node visits + 48 x leaf slots "
                                 "(binary: 64 B a visit = 32 B per box test)",
        "node_bytes_per_visit": node_bytes,
        "node_visits_per_ray": round(counts["nodes_per_ray"], 3),
        "box_tests_per_ray": round(box_tests, 3),
        "slots_per_ray": round(counts["slots_per_ray"], 3),
        "rays_per_launch": N_RAYS,
        "kernel_ms": round(closest_s * 1e3, 4),
        "hbm_peak": hbm_peak, "hbm_peak_source": peak_kind,
        "frac_of_hbm": round(achieved / hbm_peak, 4)})
    # the same kernel with 32 B counted per node visit, whatever the layout
    # reads (B_ray = 32 + 8 + 32 N_nodes + 48 N_prims)
    per_visit32 = 32 + 8 + 32 * counts["nodes_per_ray"] + 48 * counts["slots_per_ray"]
    ach32 = per_visit32 * N_RAYS / closest_s / 1e9
    roof["per_node_32B"] = {"algorithmic_bytes_per_ray": round(per_visit32, 1),
                            "achieved": round(ach32, 1),
                            "frac": round(ach32 / roof["peak"], 4)}

    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            rate, cores, dt, sample, kd = cpu_oracle_rate(soup, rays, ra, args.cpu_rays)
            cpu = {"value": round(rate, 3), "unit": "Mrays/s", "cores": cores, "kind": "port",
                   "sample": sample, "kdtree": kd}
        line = {
            "metric": "Mrays/s", "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(total_s * 1e3 / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args, world),
            "e2e": e2e,
            "roofline": roof,
            "cpu_baseline": cpu,
            "gpu_launches": 2 * args.steps,
            "clocks": clk.summary(),
            "closest_ms": round(float(np.mean(closest_ms)), 4),
            "any_ms": round(float(np.mean(any_ms)), 4),
            "hit_fraction": round(hit_frac, 4),
            "bvh_build_ms": round(st["bvh_build_ms"], 1),
            "bvh_nodes": st["bvh_nodes"],
            "path_integrator": render,
            "light_tracer": light,
            "sppm": sppm,
            "batched_wavefront": batched,
            "serving": served,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def traversal_counts(g, rays):
    """Nodes visited and leaf slots tested per closest-hit ray, counted by the
    instrumented traversal (depth-first, each leaf tested when reached) on the
    first 1M rays."""
    try:
        return g.traversal_counts(np.ascontiguousarray(rays[:, : 1 << 20]))
    except AttributeError:
        return {"nodes_per_ray": float("nan"), "slots_per_ray": float("nan")}


def profile_traffic():
    """DRAM bytes per k_trace_closest launch from the committed ncu summary."""
    p = ROOT / "profiles" / "trace_closest_soup1m.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return None
    return None


def run_batch_profile(args):
    """Plain per-job passes against one batch over the same jobs, for
    profiling: `--batch-profile N` instances of the batched workload (seed 5),
    the batch with 4M slots and one CUDA graph per iteration (no autotuning).
    `--batch-profile-mode` picks "plain", "batched" or "both"."""
    import torch

    from bling_gb300 import build as gb
    gb.build()
    from bling_gb300 import scene as S
    from bling_gb300.api import Batch, Context
    from bling_gb300.autotune import extent_samples
    inst = S.batch_instances(n=args.batch_profile, seed=5)
    ctx = Context(device=0)
    gs = [ctx.scene(i.scene) for i in inst]
    params = [i.params for i in inst]
    films = [ctx.film(p.width, p.height) for p in params]
    samples = sum(extent_samples(p) for p in params)
    out = {"workload": f"batched workload, {len(inst)} instances (seed 5)", "path_samples": samples,
           "triangles": sum(i.n_tris for i in inst)}
    if args.batch_profile_mode in ("plain", "both"):
        gs[0].render_pass(films[0], params[0], 0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for g, p, f in zip(gs, params, films):
            g.render_pass(f, p, 1)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out["plain"] = {"s": round(dt, 3), "path_samples_per_s": round(samples / dt, 1)}
    if args.batch_profile_mode in ("batched", "both"):
        b = Batch(ctx, slots=1 << 22, graph_mode=1)
        b.submit(gs[0], films[0], params[0], 0)
        b.run()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for g, p, f in zip(gs, params, films):
            b.submit(g, f, p, 1)
        b.run()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out["batched"] = {"s": round(dt, 3), "path_samples_per_s": round(samples / dt, 1),
                          "iterations": b.stats()["iterations"]}
        b.close()
    print(json.dumps(out), flush=True)
    ctx.close()


def main():
    global N_RAYS, N_ANY
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-rays", type=int, default=CPU_SAMPLE_RAYS)
    ap.add_argument("--full-rays", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-render", action="store_true", help="skip the path-integrator workloads")
    ap.add_argument("--no-heightfield", action="store_true")
    ap.add_argument("--wide-bvh", action="store_true", help="8-wide quantised BVH layout")
    ap.add_argument("--compact-bvh", action="store_true",
                    help="32-byte quantised binary BVH nodes")
    ap.add_argument("--gpu-bvh", action="store_true", help="build the BVH on the GPU")
    ap.add_argument("--bin-rays", action="store_true",
                    help="path integrator: Morton-ordered bounce rays")
    ap.add_argument("--no-light", action="store_true", help="skip the light-tracer workload")
    ap.add_argument("--light-photons", type=int, default=1 << 22)
    ap.add_argument("--light-profile", action="store_true",
                    help="only run light passes of the Cornell room (profiling)")
    ap.add_argument("--no-sppm", action="store_true", help="skip the SPPM workload")
    ap.add_argument("--sppm-photons", type=int, default=1 << 20)
    ap.add_argument("--sppm-profile", action="store_true",
                    help="only run SPPM passes of the Cornell room (profiling)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched workload")
    ap.add_argument("--batch-instances", type=int, default=64)
    ap.add_argument("--no-serving", action="store_true", help="skip the serving workload")
    ap.add_argument("--serving-jobs", type=int, default=32)
    ap.add_argument("--serving-iters", type=int, default=4,
                    help="wavefront iterations between admission rounds")
    ap.add_argument("--render-size", type=int, nargs=3, metavar=("W", "H", "STRATA"),
                    help="only render the large-mesh workload at W x H, STRATA^2 spp (profiling)")
    ap.add_argument("--batch-profile", type=int, default=0, metavar="N",
                    help="only time plain passes against one batch over N batched-workload "
                         "instances (profiling)")
    ap.add_argument("--batch-profile-mode", default="both", choices=["plain", "batched", "both"])
    ap.add_argument("--rays", type=int, default=N_RAYS,
                    help="closest-hit rays per step (any-hit: half); smaller for profiling")
    args = ap.parse_args()
    N_RAYS, N_ANY = args.rays, args.rays // 2
    if args.warmup < 3:
        args.warmup = 3
    if args.light_profile:
        run_light_profile(args)
    elif args.sppm_profile:
        run_sppm_profile(args)
    elif args.render_size:
        run_render_profile(args)
    elif args.batch_profile:
        run_batch_profile(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
