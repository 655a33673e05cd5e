"""Build the CUDA library and the drop-in executable in-tree with nvcc.

Outputs (git-ignored):
  tcsem_fdtd_gb300/libtcsem.so   -- the C-ABI library of include/tcsem.h
  tcsem_fdtd_gb300/tcsem_fdtd    -- drop-in replacement of the reference executable
  tcsem_fdtd_gb300/libtcsem_check.so -- (build_check) the same library with every global
                                    access of the kernels bounds-checked (-DTCSEM_CHECK)
Every translation unit is compiled for sm_103a only, in parallel.
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
LIB = os.path.join(PKG, "libtcsem.so")
BUILD_CHECK = os.path.join(PKG, "_build_check")
LIB_CHECK = os.path.join(PKG, "libtcsem_check.so")
CLI = os.path.join(PKG, "tcsem_fdtd")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["setup.cpp", "volume.cu", "boundary.cu", "rx.cu", "sim.cu", "batch.cu", "persist.cu"]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
                   "-I", CSRC, "--expt-relaxed-constexpr"]


def _compile(src, verbose, check=False):
    obj = os.path.join(BUILD_CHECK if check else BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(ROOT, "include", "tcsem.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) > os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc()] + _flags() + (["-DTCSEM_CHECK"] if check else []) + ["-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd[1:1] = ["-x", "cu"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"], check=True)
        os.replace(tmp, LIB)
    cli_obj = _compile("cli.cpp", verbose)
    if not os.path.exists(CLI) or os.path.getmtime(CLI) < max(os.path.getmtime(LIB), os.path.getmtime(cli_obj)):
        subprocess.run([nvcc()] + ARCH + ["-o", CLI, cli_obj, "-L", PKG, "-ltcsem", "-Xlinker", "-rpath=$ORIGIN"],
                       check=True)
    return LIB


def build_check(verbose=False, jobs=None):
    """The library with bounds-checked kernels (check.cuh): an index outside its array is
    recorded in the device error word and the access skipped."""
    os.makedirs(BUILD_CHECK, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, check=True), SOURCES))
    if not os.path.exists(LIB_CHECK) or any(os.path.getmtime(o) > os.path.getmtime(LIB_CHECK) for o in objs):
        tmp = LIB_CHECK + f".tmp{os.getpid()}"
        subprocess.run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"], check=True)
        os.replace(tmp, LIB_CHECK)
    return LIB_CHECK


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
