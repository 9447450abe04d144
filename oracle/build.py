"""Build recipe for the CPU oracle shared library (test infrastructure only).

Compiles ``bem_oracle.cpp`` with g++ (C++17, OpenMP, -O3, no host-specific
-march so the same recipe works on x86_64 and aarch64) into
``oracle/_build/liboracle.so``.  The reference engine is Julia and has no C/C++
sources, so there is no ``oracle/_ref`` build.
"""

from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SOURCE = HERE / "bem_oracle.cpp"
BUILD_DIR = HERE / "_build"
LIBRARY = BUILD_DIR / "liboracle.so"


def build_oracle(force: bool = False) -> Path:
    BUILD_DIR.mkdir(exist_ok=True)
    if not force and LIBRARY.exists() and LIBRARY.stat().st_mtime >= SOURCE.stat().st_mtime:
        return LIBRARY
    tmp = LIBRARY.with_suffix(f".so.tmp{os.getpid()}")
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp), str(SOURCE)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build_oracle(force=True))
