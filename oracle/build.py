"""Build the CPU oracle (test infrastructure): oracle/_build/liboracle.so.

Plain g++, -O2, OpenMP when the compiler supports it. The oracle is the checker for the CUDA
path; only tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
"""
from __future__ import annotations

import pathlib
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"
SRCS = sorted(HERE.glob("*.cpp"))
HDRS = sorted(HERE.glob("*.h")) + [HERE.parent / "include" / "sty_gb300.h"]


def build(verbose: bool = False, force: bool = False) -> pathlib.Path:
    OUT.mkdir(exist_ok=True)
    if not force and LIB.exists():
        t = LIB.stat().st_mtime
        if all(p.stat().st_mtime <= t for p in [*SRCS, *HDRS]):
            return LIB
    # no FMA contraction: the geometric tests restate the reference's separate f32 mul/add
    base = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(LIB), *map(str, SRCS)]
    for extra in (["-fopenmp"], []):
        cmd = base[:1] + extra + base[1:]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode == 0:
            return LIB
        err = r.stderr
    raise RuntimeError(f"oracle build failed:\n{err}")


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
