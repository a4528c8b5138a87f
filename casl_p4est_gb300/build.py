"""Build the native library ``liblsgpu.so`` in-tree.

Host C++ (grid, flattener, drivers, C ABI) is compiled with g++ and ``-ffp-contract=off`` so that the
grid geometry and every precomputed coefficient round exactly as the reference's plain double
expressions on both x86_64 and aarch64. CUDA sources are compiled for sm_103a only; the FP64 kernels
additionally with ``-fmad=false`` (no contracted multiply-adds).

Usage: ``python -m casl_p4est_gb300.build`` (or ``build()`` from Python).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liblsgpu.so")

HOST_SOURCES = ["forest.cpp", "tables.cpp", "tables32.cpp", "level_set.cpp", "capi.cpp", "io.cpp"]
CUDA_SOURCES = {"kernels_fp64.cu": ["-fmad=false"], "kernels_interp.cu": ["-fmad=false"], "kernels_mixed.cu": [], "noalloc.cu": [],
                "flatten.cu": ["-fmad=false"]}
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home() -> str:
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if home and os.path.isdir(home):
        return home
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile and link liblsgpu.so; returns its path."""
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".hpp", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "lsgpu.h"))
    jobs = []
    objs = []
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                         "-I" + os.path.join(cuda, "include"), "-c", s, "-o", o])
    for src, extra in CUDA_SOURCES.items():
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            jobs.append([nvcc, GENCODE, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", *extra, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    if force or jobs or _newer(LIB, objs):
        tmp = LIB + ".tmp"
        _run(["g++", "-shared", "-fopenmp", "-o", tmp, *objs, "-L" + os.path.join(cuda, "lib64"), "-lcudart_static", "-lpthread",
              "-ldl", "-lrt", "-Wl,-rpath," + os.path.join(cuda, "lib64")])
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
