"""Build libhsr.so (CUDA kernels for sm_103a + the C ABI) in-tree with nvcc.

Each translation unit is compiled in parallel, then linked with the static CUDA runtime.
Device code keeps IEEE semantics: no FMA contraction (--fmad=false), correctly rounded
division and square root, denormals preserved; host code is built with
-ffp-contract=off so host-side matrix products round like the reference.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(OUT_DIR, "libhsr.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

SOURCES = ["hsr_runtime.cu", "kernels_geom.cu", "kernels_bin.cu", "kernels_raster.cu", "hsr_noalloc.cu", "hsr_serve.cu",
           "hsr_io.cu", "hsr_uniforms.cpp"]

NVCC_FLAGS = [ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "--prec-div=true", "--prec-sqrt=true",
              "--ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2,-fvisibility=hidden",
              "-DHSR_BUILD"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "hsr.h")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    cmd = [nvcc(), ARCH, "-shared", "-o", LIB, *objs, "-cudart=static", "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force=True))
