"""Builds the CUDA library in-tree: puresoft3d_gb300/_lib/libps3d.so.

nvcc compiles each translation unit for sm_103a only, in parallel, with FMA
contraction off (--fmad=false, -ffp-contract=off on the host side) and IEEE
division / square root, so the coverage and depth chain reproduces the
reference's FP32 results bit for bit.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libps3d.so")
SOURCES = ["setup_bin.cu", "raster_shade.cu", "raster_warp.cu", "post.cu", "pipeline.cpp", "objx.cpp"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17", "--fmad=false",
         "-prec-div=true", "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
         "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def _stamp() -> float:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "ps3d.h"), __file__]
    return max(os.path.getmtime(f) for f in files)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _stamp():
        return LIB
    os.makedirs(os.path.join(OUT_DIR, "obj"), exist_ok=True)

    def compile_one(src):
        obj = os.path.join(OUT_DIR, "obj", src + ".o")
        cmd = [NVCC] + FLAGS + ["-x", "cu", "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    r = subprocess.run([NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o", tmp] + objs,
                       capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
