"""Builds the engine's shared library for sm_103a with nvcc.

Every ``csrc/*.cu`` translation unit (nvcc) and every host-only
``csrc/*.cpp`` unit (the host C++ compiler) is compiled in parallel into
``_build/`` and linked into ``everett_gb300/libeverett_gb300.so`` (in-tree,
so the tests and the benchmark load exactly this file).  A unit is rebuilt
only when it or a header is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE.parent / "_build"
LIB = HERE / "libeverett_gb300.so"
INCLUDE = HERE.parent / "include"

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
# host units: sin and cos stay separate libm calls (no sincos fusion), as the
# reference's gate constructors make them
CXXFLAGS = ["-O2", "-fPIC", "-std=c++17", "-fno-builtin-sin", "-fno-builtin-cos"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-Xptxas", "-O3"]


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")))


def _compile(src: Path, verbose: bool) -> Path:
    obj = BUILD / (src.stem + ".o")
    newest_dep = max([src.stat().st_mtime] + [h.stat().st_mtime for h in _headers()])
    if obj.exists() and obj.stat().st_mtime >= newest_dep:
        return obj
    if src.suffix == ".cpp":
        cmd = [CXX, *CXXFLAGS, "-c", str(src), "-o", str(obj)]
    else:
        cmd = [NVCC, *ARCH, *FLAGS, "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"{cmd[0]} failed on {src.name}:\n{res.stdout}\n{res.stderr}")
    return obj


def build(verbose: bool = False) -> Path:
    """Compiles and links the engine; returns the library path."""
    BUILD.mkdir(exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if LIB.exists() and LIB.stat().st_mtime >= max(o.stat().st_mtime for o in objs):
        return LIB
    cmd = [NVCC, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
