"""Builds libdwgb.so (all CUDA sources, sm_103a) in-tree with nvcc.

Each translation unit is compiled in parallel, then linked into one shared library next to
the sources (deeperwin_gb300/csrc/libdwgb.so). No CMake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

CSRC = Path(__file__).resolve().parent / "csrc"
BUILD = CSRC / "_build"
LIB = CSRC / "libdwgb.so"
SOURCES = ["model.cu", "net.cu", "gemm_simt.cu", "gemm_tc.cu", "det.cu", "mcmc.cu", "api.cu", "backward.cu", "noalloc.cu", "fp64.cu", "guard.cu", "forces.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _flags(verbose: bool):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                "-I", str(CSRC), "-I", str(CSRC.parent.parent / "include")]
    if verbose:
        f += ["-Xptxas", "-v"]
    return f


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = [CSRC / s for s in SOURCES if (CSRC / s).exists()]
    headers = list(CSRC.glob("*.cuh")) + [CSRC.parent.parent / "include" / "dwgb.h"]
    newest_hdr = max(h.stat().st_mtime for h in headers)
    objs = []
    jobs = []
    for s in srcs:
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if force or not o.exists() or o.stat().st_mtime < max(s.stat().st_mtime, newest_hdr):
            jobs.append([nvcc(), *_flags(verbose), "-c", str(s), "-o", str(o)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError(f"nvcc failed: {' '.join(cmd)}")
    if force or jobs or not LIB.exists():
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
