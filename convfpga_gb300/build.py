"""Builds libconvgpu.so in-tree: the CUDA kernels and runtime for sm_103a plus the C ABI.

    python -m convfpga_gb300.build        (or convfpga_gb300.build.build())

Translation units compile in parallel into convfpga_gb300/_build/ and link into
convfpga_gb300/libconvgpu.so. A unit is rebuilt when it or any header under csrc/ or
include/ is newer than its object.
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
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libconvgpu.so")
APP_SRC = os.path.join(PKG, "app", "convolution.cpp")
APP = os.path.join(PKG, "convolution")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"] + ARCH
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wextra"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers_mtime() -> float:
    m = 0.0
    for d in (CSRC, INCLUDE):
        for dp, _, fs in os.walk(d):
            for f in fs:
                if f.endswith((".h", ".cuh", ".hpp")):
                    m = max(m, os.path.getmtime(os.path.join(dp, f)))
    return m


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if src.endswith(".cu"):
        cmd = [_nvcc(), *NVCC_FLAGS, "-I", CSRC, "-I", INCLUDE, "-c", src, "-o", obj]
    else:
        cmd = [os.environ.get("CXX", "g++"), *CXX_FLAGS, "-I", CSRC, "-I", INCLUDE, "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stderr.strip() or r.stdout.strip()):
        print(r.stdout, r.stderr, flush=True)
    return obj


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdr = _headers_mtime()
    srcs = sources()
    todo = []
    for s in srcs:
        obj = os.path.join(BUILD, os.path.basename(s) + ".o")
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(s), hdr):
            todo.append(s)
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda s: _compile(s, verbose), todo))
    objs = [os.path.join(BUILD, os.path.basename(s) + ".o") for s in srcs]
    if todo or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    build_app(verbose)
    return LIB


def build_app(verbose: bool = False) -> str:
    """The `convolution` sample application, linked against libconvgpu.so (rpath $ORIGIN)."""
    if os.path.exists(APP) and os.path.getmtime(APP) >= max(os.path.getmtime(APP_SRC), os.path.getmtime(LIB)):
        return APP
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-Wall", "-I", INCLUDE, APP_SRC, "-o", APP,
           "-L", PKG, "-lconvgpu", "-Wl,-rpath,$ORIGIN", "-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"app build failed\n{r.stdout}\n{r.stderr}")
    return APP


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
