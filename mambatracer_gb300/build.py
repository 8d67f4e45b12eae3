"""Build libmambatracer.so (the C-ABI library) in-tree with nvcc for sm_103a.

Each CUDA translation unit compiles in parallel to an object under _build/,
then nvcc links the shared library next to this file. FMA contraction is off in
device and host code so that traversal and shading arithmetic keep the
reference kernels' operation order (division and sqrt stay IEEE-rounded, the
nvcc default).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(os.path.dirname(HERE), "_build")
LIB = os.path.join(HERE, "libmambatracer.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["mt_api.cu", "mt_kernels.cu", "mt_env.cu", "mt_compact.cu", "mt_job.cu", "mt_image.cu", "mt_server.cu", "mt_plain.cu", "mt_preview.cu", "mt_bvh.cu", "mt_obj.cpp", "mt_batch.cu", "mt_wide.cu"]


def nvcc() -> str:
    for p in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if p and os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return [*ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
            "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", os.path.join(os.path.dirname(HERE), "include"), *extra]


def _compile(src: str, verbose: bool, ptxas_v: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj, *_flags(["-Xptxas", "-v"] if ptxas_v else [])]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if verbose or r.returncode:
        sys.stderr.write(r.stderr)
    if r.returncode:
        raise RuntimeError(f"nvcc failed on {src}")
    return obj


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "mambatracer.h"))
    deps.append(__file__)
    newest = max(os.path.getmtime(p) for p in deps)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) > newest:
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, ptxas_v), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", *ARCH, "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        sys.stderr.write(r.stderr)
        raise RuntimeError("link failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, ptxas_v="--ptxas" in sys.argv))
