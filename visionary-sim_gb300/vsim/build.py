"""Builds libvsim.so in-tree for sm_103a (GB300), and the CPU oracle.

The library is compiled straight with nvcc, one translation unit per
process in parallel, then linked into ``vsim/libvsim.so`` next to this
file. Every kernel file is compiled with ``-fmad=false`` and the host code
with ``-ffp-contract=off``: each multiply and add rounds on its own, the
evaluation the solver's results are defined by.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
CSRC = PACKAGE.parent / "csrc"
INCLUDE = PACKAGE.parent.parent / "include"
BUILD = PACKAGE.parent / "_build"
LIB = PACKAGE / "libvsim.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "-fmad=false", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", f"-I{INCLUDE}",
]
SOURCES = ["host.cpp", "sim.cu", "server.cu", "step_kernels.cu", "colour_tma.cu", "session.cu", "splat_sort.cu", "grab.cu",
           "cloud_volume.cu"]


def nvcc() -> str:
    found = shutil.which("nvcc")
    if found:
        return found
    candidate = Path("/usr/local/cuda/bin/nvcc")
    if candidate.exists():
        return str(candidate)
    raise RuntimeError("nvcc not found: libvsim cannot be built")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [INCLUDE / "vsim.h"]


def build_library(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile libvsim.so if any source is newer than it; returns its path."""
    BUILD.mkdir(exist_ok=True)
    compiler = nvcc()
    headers = _headers()
    objects = []
    jobs = []
    for src in SOURCES:
        path = CSRC / src
        obj = BUILD / (src + ".o")
        objects.append(obj)
        if force or _stale(obj, [path] + headers):
            cmd = [compiler, *ARCH, *NVCC_FLAGS, *(extra or []), "-c", str(path), "-o", str(obj)]
            jobs.append(cmd)

    def run(cmd: list[str]) -> str:
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
        return proc.stdout + proc.stderr

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as pool:
            for out in pool.map(run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or jobs or _stale(LIB, objects):
        tmp = LIB.with_suffix(".so.tmp")
        run([compiler, *ARCH, "-shared", "-o", str(tmp), *map(str, objects)])
        os.replace(tmp, LIB)
    return LIB


def build_oracle(force: bool = False) -> Path:
    """Compile the CPU oracle (test infrastructure) with its Makefile."""
    oracle = PACKAGE.parent.parent / "oracle"
    target = oracle / "_build" / "libvsim_oracle.so"
    if force and target.exists():
        target.unlink()
    proc = subprocess.run(["make", "-C", str(oracle), "-s"], capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{proc.stdout}\n{proc.stderr}")
    return target


if __name__ == "__main__":
    import sys

    print(build_library(force="--force" in sys.argv, verbose=True))
    print(build_oracle())
