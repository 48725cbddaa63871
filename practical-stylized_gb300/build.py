"""Build libsty_gb300.so (the CUDA product library) in-tree.

Every .cu file under csrc/ is compiled for sm_103a only, in parallel, and linked into
lib/libsty_gb300.so. Nothing here depends on PyTorch. Run directly (`python build.py`) or via
`__graft_entry__.build()`.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "lib"
OBJ = PKG / "_build"
LIB = OUT / "libsty_gb300.so"
# the same objects as a static archive, for a host that links the library into its own binary
# (the reference's Rust build links its C++ extension statically); link with -lcudart -lstdc++
STATIC = OUT / "libsty_gb300.a"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
    # host code: no FMA contraction (the camera frame and other host-side set-up round the same way on
    # x86-64 and Arm hosts)
    "-Xcompiler", "-ffp-contract=off",
    "-I", str(ROOT / "include"), "-I", str(CSRC),
]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _newer(dst: pathlib.Path, srcs) -> bool:
    if not dst.exists():
        return False
    t = dst.stat().st_mtime
    return all(pathlib.Path(s).stat().st_mtime <= t for s in srcs)


def build(verbose: bool = False, force: bool = False) -> pathlib.Path:
    nvcc = _nvcc()
    OUT.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "sty_gb300.h"]

    def compile_one(src: pathlib.Path) -> pathlib.Path:
        obj = OBJ / (src.stem + ".o")
        if not force and _newer(obj, [src, *headers]):
            return obj
        cmd = [nvcc, *NVFLAGS, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(sources))) as ex:
        objs = list(ex.map(compile_one, sources))
    if force or not _newer(LIB, objs):
        # -z defs: an unresolved symbol fails the link here, not the first load of the library
        cmd = [nvcc, *ARCH, "-shared", "-Xlinker", "-z", "-Xlinker", "defs", "-o", str(LIB), *map(str, objs)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if force or not _newer(STATIC, objs):
        if STATIC.exists():
            STATIC.unlink()
        cmd = [nvcc, *ARCH, "-lib", "-o", str(STATIC), *map(str, objs)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"archive failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
