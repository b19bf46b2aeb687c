"""Build libaxgb.so for sm_103a, in tree (helm-project_gb300/axgb/lib/).

CUDA translation units are compiled by nvcc with one -gencode
(compute_103a -> sm_103a); the geometry units (prep.cu, weights.cu,
coastal.cu, nearest.cu, bilinear.cu) with --fmad=false so double expressions, and the
float distances of the nearest searches, round as written. The host C++ units
(api.cpp, esmf_io.cpp) are compiled by g++ with -ffp-contract=off and OpenMP
(parallel sort in the grid detector). Units compile in parallel; the link uses nvcc.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUTDIR = os.path.join(HERE, "axgb", "lib")
OBJDIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUTDIR, "libaxgb.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")

UNITS = [
    ("prep.cu", ["--fmad=false"]),
    ("weights.cu", ["--fmad=false"]),
    ("apply.cu", []),
    ("staged.cu", []),
    ("scan_sort.cu", []),
    ("coastal.cu", ["--fmad=false"]),
    ("nearest.cu", ["--fmad=false"]),
    ("bilinear.cu", ["--fmad=false"]),
]
HOST_UNITS = ["api.cpp", "esmf_io.cpp"]  # host C++ (g++)
HEADERS = ["internal.hpp", "geom.cuh", "fp32x2.cuh", "lbvh.cuh", "gather_schedule.hpp", os.path.join("..", "..", "include", "axgb.h")]


def _nvcc():
    p = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
    return p


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUTDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS]
    jobs = []
    objs = []
    for src, extra in UNITS:
        srcp = os.path.join(CSRC, src)
        obj = os.path.join(OBJDIR, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [srcp, *hdrs, __file__]):
            cmd = [_nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++20", "-Xcompiler", "-fPIC", "-Xcompiler",
                   "-ffp-contract=off", *extra, "-c", srcp, "-o", obj]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in HOST_UNITS:
        srcp = os.path.join(CSRC, src)
        obj = os.path.join(OBJDIR, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [srcp, *hdrs, __file__]):
            jobs.append(["g++", "-std=c++20", "-O2", "-fPIC", "-ffp-contract=off", "-fopenmp",
                         "-I", os.path.join(CUDA_HOME, "include"), "-c", srcp, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        outs = list(ex.map(_compile, jobs))
    if verbose:
        for o in outs:
            sys.stderr.write(o)
    if jobs or not os.path.exists(LIB):
        link = [_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lgomp"]
        _compile(link)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
