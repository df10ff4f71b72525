"""Builds the native library horses3d_gb300/lib/libhorses3d_gb300.so in the source tree.

Host C++ (mesh, geometry, spectral operators) is compiled with g++; the CUDA kernels and the C ABI
with nvcc for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``). Translation units are
compiled in parallel and only when their sources changed. No CPU fallback is built.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_objs"
LIB = PKG / "lib" / "libhorses3d_gb300.so"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O2", "-fPIC", "-fopenmp", "-std=c++17", "-Wall", f"-I{INCLUDE}"]
NVCCFLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
             f"-I{INCLUDE}", *ARCH]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build horses3d_gb300")
    return cand


def _deps(src: Path):
    if src.suffix == ".cu":
        return [src, *sorted((CSRC / "cuda").glob("*.cuh")), *sorted((CSRC / "host").glob("*.hpp")),
                INCLUDE / "horses3d_gb300.h"]
    return [src, *sorted((CSRC / "host").glob("*.hpp")), INCLUDE / "horses3d_gb300.h"]


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


# The FP32 (mixed-form) kernels use the fast single-precision division/sqrt and flush denormals;
# the FP64 translation units keep IEEE arithmetic.
FAST_FP32_UNITS = {"dg_inst_fp32.cu", "dg_var_fp32.cu"}


def _compile(src: Path) -> Path:
    out = OBJ / (src.stem + (".cu.o" if src.suffix == ".cu" else ".o"))
    if not _stale(out, _deps(src) + [Path(__file__)]):
        return out
    if src.suffix == ".cu":
        extra = ["--use_fast_math"] if src.name in FAST_FP32_UNITS else []
        cmd = [_nvcc(), *NVCCFLAGS, *extra, "-c", str(src), "-o", str(out)]
    else:
        cmd = [os.environ.get("CXX", "g++"), *CXXFLAGS, "-c", str(src), "-o", str(out)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return out


def build(verbose: bool = False) -> Path:
    OBJ.mkdir(parents=True, exist_ok=True)
    LIB.parent.mkdir(parents=True, exist_ok=True)
    sources = sorted((CSRC / "host").glob("*.cpp")) + sorted((CSRC / "cuda").glob("*.cu"))
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, sources))
    if _stale(LIB, objs):
        cmd = [_nvcc(), "-shared", *ARCH, "-o", str(LIB), *map(str, objs), "-Xcompiler", "-fopenmp", "-lgomp"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
