"""Build the GB300 path-tracing core: bling_gb300/libbling_gpu.so.

CUDA translation units are compiled for sm_103a only, in parallel, with
``-fmad=false`` so that intersection and shading arithmetic rounds exactly
like the reference's (no contracted multiply-adds); host code is compiled with
``-ffp-contract=off`` for the same reason.  The CUDA runtime is linked
statically, so the library only needs the driver at run time.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libbling_gpu.so"
PROBE_LIB = PKG / "libbling_probe.so"  # measurement only: the L2 bandwidth probe
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SRCS = ["api.cu", "kernels_trace.cu", "integrator.cu", "scene_upload.cu", "batch.cu",
           "server.cu", "lighttrace.cu", "sppm.cu", "bvh_gpu.cu"]
CPP_SRCS = ["bvh.cpp"]
PROBE_SRCS = ["l2probe.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    """Every header of csrc/ (any source may include any of them), the public
    header and this recipe."""
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh"))
    return headers + [PKG.parent / "include" / "bling_gpu.h", Path(__file__)]


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    m = obj.stat().st_mtime
    return any(p.stat().st_mtime > m for p in [src, *_deps()])


def _compile(src: Path, obj: Path, verbose_ptxas: bool):
    if src.suffix == ".cu":
        cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
               "-Xcompiler", "-fPIC,-O2,-ffp-contract=off,-pthread",
               "-I", str(CSRC), "-I", str(PKG.parent / "include"), "-c", str(src), "-o", str(obj)]
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off",
               "-I", str(CSRC), "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stderr


def _link(lib: Path, objs, changed: bool):
    if changed or not lib.exists() or any(o.stat().st_mtime > lib.stat().st_mtime for o in objs):
        tmp = lib.with_suffix(f".{os.getpid()}.tmp.so")
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs),
               "-Xcompiler", "-pthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    jobs = []
    for name in CU_SRCS + CPP_SRCS + PROBE_SRCS:
        src = CSRC / name
        obj = BUILD / (name + ".o")
        if force or verbose_ptxas or _stale(obj, src):
            jobs.append((src, obj))
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            logs = list(ex.map(lambda j: _compile(j[0], j[1], verbose_ptxas), jobs))
    _link(LIB, [BUILD / (n + ".o") for n in CU_SRCS + CPP_SRCS], bool(jobs))
    _link(PROBE_LIB, [BUILD / (n + ".o") for n in PROBE_SRCS], bool(jobs))
    if verbose_ptxas:
        for log in logs:
            print(log)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
