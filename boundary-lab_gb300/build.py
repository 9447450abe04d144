"""Build recipe for the GB300 BEM shared library (libgb300_bem.so).

Compiles every CUDA translation unit for sm_103a only (one -gencode, no PTX
fallback) and the host planner with g++, in parallel, then links one shared
library into ``_build/``.  No cmake; the same recipe runs on x86_64 and on
aarch64 hosts (no host-specific flags).
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIBRARY = BUILD / "libgb300_bem.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["bem_assembly.cu", "bem_lu.cu", "bem_lu_cluster.cu", "bem_gemm_tc.cu", "bem_field.cu", "bem_capi.cu",
                "bem_noalloc.cu"]
CXX_SOURCES = ["bem_plan.cpp"]
HEADERS = ["bem_common.cuh", "bem_internal.h", "bem_kernels.h"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 BEM library needs the CUDA toolkit to build")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = [CSRC / h for h in HEADERS] + [HERE.parent / "include" / "gb300_bem.h"]
    jobs = []
    objects = []
    for src in CUDA_SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        objects.append(obj)
        if force or _stale(obj, [CSRC / src, *headers]):
            cmd = [nvcc, "-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-c", str(CSRC / src),
                   "-o", str(obj)]
            if verbose_ptxas:
                cmd[1:1] = ["-Xptxas", "-v"]
            jobs.append(cmd)
    for src in CXX_SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        objects.append(obj)
        if force or _stale(obj, [CSRC / src, *headers]):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-c", str(CSRC / src), "-o", str(obj)])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as pool:
            results = list(pool.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, res in zip(jobs, results):
            if verbose_ptxas and res.stderr:
                print(res.stderr)
            if res.returncode != 0:
                raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if force or jobs or _stale(LIBRARY, objects):
        tmp = LIBRARY.with_suffix(f".so.tmp{os.getpid()}")
        cmd = [nvcc, "-shared", *ARCH, "-o", str(tmp), *map(str, objects), "-lcublas", "-lpthread"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
