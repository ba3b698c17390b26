"""Builds libima2p_gb300.so in-tree from ima2p_gb300/csrc/*.cu for sm_103a.

Every translation unit is compiled by nvcc in parallel, then linked into one
shared library next to this file.  No torch extension machinery is involved:
the library is a plain C ABI (include/ima_gpu.h).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libima2p_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# k_treeweight.cu, k_popmig.cu and k_updgen.cu restate the reference's FP64
# arithmetic term by term: without FMA contraction it rounds as the host's does
NOFMAD_FILES = {"k_treeweight.cu", "k_popmig.cu", "k_updgen.cu"}
NOFMAD = ["-fmad=false"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + os.path.join(ROOT, "include")]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _stale(src, obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + deps)


def build_library(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    deps = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    exe = nvcc()
    jobs = []
    objs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or _stale(s, o, deps):
            extra = NOFMAD if os.path.basename(s) in NOFMAD_FILES else []
            jobs.append([exe] + ARCH + FLAGS + extra + ["-c", s, "-o", o])

    def run(cmd):
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
        if verbose:
            print(" ".join(cmd[-3:]))
        return p

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        run([exe] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build_library(verbose=True))
