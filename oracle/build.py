"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/oracle.cpp into oracle/_build/liboracle.so with the
arithmetic flags the restatement relies on: IEEE binary32 without operation
contraction (-ffp-contract=off), no fast-math.  Used by tests/, by
__graft_entry__.build() and by bench.py's CPU-baseline leg.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "liboracle.so"
SRCS = [HERE / "oracle.cpp"]
DEPS = SRCS + [HERE / "oracle.h", HERE / "oracle_math.h", HERE / "kdtree.h",
               HERE.parent / "include" / "bling_gpu.h",
               HERE.parent / "bling_gb300" / "csrc" / "spectrum_tables.h"]
FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
         "-fno-fast-math", "-Wall", "-Wno-unused-function"]


def build(force: bool = False) -> Path:
    if not force and OUT.exists():
        mtime = OUT.stat().st_mtime
        if all(p.stat().st_mtime <= mtime for p in DEPS):
            return OUT
    OUT.parent.mkdir(parents=True, exist_ok=True)
    tmp = OUT.with_suffix(f".{os.getpid()}.tmp.so")
    cmd = ["g++", *FLAGS, *map(str, SRCS), "-o", str(tmp)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
