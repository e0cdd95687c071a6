"""Build the CUDA library ``_build/libopir_gb300.so`` in-tree for sm_103a,
and the CPU client library ``_build/libopir_client.so``.

Each CUDA translation unit under ``csrc/`` is compiled by nvcc in parallel and
the objects are linked into one shared library that exports the C ABI of
``include/onionpir_gpu.h``.  No torch headers are involved: the library is a
plain CUDA/C++ shared object loadable from C, C++ or Python (ctypes).  The
client (``csrc/client.cpp``, C ABI ``include/onionpir_client.h``) is plain
C++ built by the host compiler; it needs no GPU.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libopir_gb300.so")
CLIENT_LIB = os.path.join(BUILD, "libopir_client.so")
CLIENT_SRC = os.path.join(CSRC, "client.cpp")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
                     "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build onionpirv2_gb300")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + [
        os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
        if f.endswith(".h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_client(force: bool = False, verbose: bool = False) -> str:
    """Compile the CPU client library (no CUDA)."""
    os.makedirs(BUILD, exist_ok=True)
    inc = os.path.join(ROOT, "include")
    deps = [CLIENT_SRC] + [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith((".h", ".hpp"))]
    if force or _stale(CLIENT_LIB, deps):
        cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
        tmp = CLIENT_LIB + f".tmp{os.getpid()}"
        cmd = [cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
               CLIENT_SRC, "-o", tmp]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"client build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, CLIENT_LIB)
    return CLIENT_LIB


def build(force: bool = False, verbose: bool = False) -> str:
    build_client(force, verbose)
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    hdrs = _headers()
    objs = []
    jobs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append([nv] + NVCC_FLAGS + ["-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r

    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        run([nv] + ARCH + ["-shared", "-o", tmp] + objs)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
