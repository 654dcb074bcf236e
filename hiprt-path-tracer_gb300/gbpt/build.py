"""Builds libgbpt.so in-tree from csrc/ (CUDA for sm_103a + C++ host code).

nvcc compiles every translation unit in parallel (one -gencode, arch=compute_103a,code=sm_103a)
and links a shared library with the CUDA runtime linked statically. The build is incremental:
nothing is recompiled when the library is newer than every source and header.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(ROOT, "csrc")
REPO = os.path.dirname(ROOT)
INCLUDE = os.path.join(REPO, "include")
LIB_PATH = os.path.join(PKG_DIR, "libgbpt.so")
BUILD_DIR = os.path.join(ROOT, "_build")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", ARCH, "-Xcompiler", "-fPIC,-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE]
CXX_FLAGS = ["-O2", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden", "-I", CSRC, "-I", INCLUDE]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbpt")
    return path


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "*.cpp")))
    hdr = sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
                 + glob.glob(os.path.join(INCLUDE, "*.h")))
    return cu, cpp, hdr


def up_to_date() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    cu, cpp, hdr = _sources()
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(p) <= t for p in cu + cpp + hdr + [__file__])


def _compile(src: str, extra) -> str:
    obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
    cmd = [nvcc(), "-c", src, "-o", obj] + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    cu, cpp, _ = _sources()
    jobs = [(s, NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_verbose else [])) for s in cu]
    jobs += [(s, CXX_FLAGS) for s in cpp]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        objs = list(ex.map(lambda j: _compile(*j), jobs))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc(), "-shared", ARCH, "-o", tmp] + objs + ["-cudart", "static", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    if verbose:
        print(f"built {LIB_PATH}", file=sys.stderr)
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_verbose="--ptxas-v" in sys.argv)
