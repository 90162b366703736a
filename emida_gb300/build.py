"""Builds libemida_gb.so (the sm_103a kernels and the C ABI) in-tree.

Each .cu translation unit is compiled by nvcc in parallel, then linked into
emida_gb300/libemida_gb.so next to this file.  Rebuilds only what changed.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libemida_gb.so")
CLI = os.path.join(HERE, "bin", "emida")
SOURCES = ["fused.cu", "brute_tc.cu", "staged.cu", "capi.cu", "multi.cu", "server.cu",
           "deformation.cu"]
HEADERS = ["common.cuh", "fft.cuh", "device_fit.cuh", "fused.cuh", "staged.cuh", "handle.cuh",
           "ptx.cuh", "brute_tc.cuh", "deformation.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
         "-ffp-contract=off", "-Xcompiler", "-O2", "--expt-relaxed-constexpr",
         "-I" + os.path.join(REPO, "include")]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libemida_gb.so")
    return path


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra):
    obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS] + \
        [os.path.join(REPO, "include", "emida_gb.h"), __file__]
    if _stale(obj, deps):
        cmd = [nvcc()] + ARCH + FLAGS + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose=False, extra=()):
    os.makedirs(OBJ, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra)), SOURCES))
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    build_cli()
    if verbose:
        print("built", LIB, "and", CLI)
    return LIB


def build_cli():
    """The `emida` command line (emida_gb300/cli), linked against the library."""
    src = os.path.join(HERE, "cli", "main.cpp")
    deps = [src, os.path.join(HERE, "cli", "tiff.hpp"), os.path.join(HERE, "cli", "text.hpp"), LIB,
            os.path.join(REPO, "include", "emida_gb", "gpu_offset.hpp")]
    if not _stale(CLI, deps):
        return CLI
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    cxx = shutil.which("g++") or "c++"
    cmd = [cxx, "-O2", "-std=c++17", "-pthread", "-I" + os.path.join(REPO, "include"), src, "-o", CLI,
           "-L" + HERE, "-lemida_gb", "-Wl,-rpath,$ORIGIN/.."]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed:\n{r.stdout}\n{r.stderr}")
    return CLI


if __name__ == "__main__":
    build(verbose=True)
