"""Build recipe of libtws.so (the product library) for sm_103a.

Each CUDA translation unit is compiled in parallel with nvcc, then linked into
``terrainwatersim_gb300/_build/libtws.so``.  Only one ``-gencode`` is used
(compute_103a / sm_103a).  The simulation arithmetic is written with explicit
round-to-nearest intrinsics; ``--fmad=false`` additionally keeps any other
float code free of multiply-add contraction, and host code is compiled with
``-ffp-contract=off`` so that x86 and Arm hosts agree.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libtws.so")

SOURCES = ["tws_step.cu", "tws_stream.cu", "tws_sweep.cu", "tws_resident.cu", "tws_aux.cu",
           "tws_export.cu",
           "tws_capi.cu",
           "tws_serve.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtws.so")


def common_flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler",
                   "-fPIC,-ffp-contract=off,-fvisibility=hidden", "-I", os.path.join(ROOT, "include")]


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, force: bool = False, extra_flags=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "tws.h"))
    cc = nvcc()

    def compile_one(src):
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        if not force and _newer(o, [s, __file__] + headers):
            return o
        cmd = [cc] + common_flags() + list(extra_flags) + ["-c", s, "-o", o]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return o

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or not _newer(LIB, objs):
        cmd = [cc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-ldl", "-lrt",
                                                            "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
