"""Build ``_build/libtbgpu.so`` from ``csrc/*.cu`` with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked into one shared
library with a C-ABI (include/tbgpu.h).  No CMake, no torch extension.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
SRC_DIR = os.path.join(PKG_DIR, "csrc")
OUT_DIR = os.path.join(PKG_DIR, "_build")
LIB = os.path.join(OUT_DIR, "libtbgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code keeps IEEE evaluation order (no a*b+c contraction into FMA, which
# gcc does by default on aarch64), as the Rust reference does.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr"] + ARCH


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OUT_DIR, os.path.basename(src).replace(".cu", ".o"))
    cmd = [nvcc(), "-c", src, "-o", obj] + NVCC_FLAGS + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build_library(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(SRC_DIR, "*.cu")))
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build_library(verbose=True, extra=sys.argv[1:])
