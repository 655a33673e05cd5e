"""Build recipe for the reference-derived checkers under oracle/_ref/.

TEST INFRASTRUCTURE.  Compiles, from the reference source tree where it lies
(TCSEM_REFERENCE_DIR, else the recipe's default location below):

* oracle/_ref/ref_host -- the reference's host setup files (ModelingSetup.cpp,
  SourceWave.cpp, ModelGridMapping.cpp, LoadRxTxPos.cpp, logspace.cpp,
  AuxiliaryMemory.cpp) linked with oracle/ref_host_driver.cpp; it writes the
  setup arrays the reference computes for a survey directory;
* oracle/_ref/ref_cpu_remap -- the reference's CPU spline remap
  (SplineGridConvIR2R_cpu.cpp) with the host setup files and
  oracle/ref_cpu_remap_driver.cpp, timed as a CPU baseline;
* oracle/_ref/<name>.cubin -- the reference's device code, unmodified, in its
  default FP64 build, compiled for sm_103a as device-only modules (no host
  code, so they load on any host): ElectricalFiled.cu, Bderivate.cu,
  SplineGridConvIR2R.cu, UpContinuation_gpu.cu, EFInterp2Rx.cu and
  initialize_UpCont_gpu_resources.cu.  oracle/ref_gpu.py drives them.

The only additions are out-of-tree shims: oracle/shim/fftw3.h (FFTW is not
installed; only its type names are needed), -Dpow10=exp10 (glibc dropped
pow10) and -DdeviceOverlap=asyncEngineCount (a device property CUDA removed).
Nothing is copied out of the reference tree; only the built files land in
oracle/_ref/ (git-ignored).  When the tree is absent the builds are skipped and
the committed golden fixtures are used instead.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REFERENCE_DIR = "/root/reference"  # where this recipe finds the reference tree by default
REF = os.environ.get("TCSEM_REFERENCE_DIR", DEFAULT_REFERENCE_DIR)
OUT = os.path.join(HERE, "_ref")

HOST_SOURCES = ["ModelingSetup.cpp", "SourceWave.cpp", "ModelGridMapping.cpp",
                "LoadRxTxPos.cpp", "logspace.cpp", "AuxiliaryMemory.cpp"]
DEVICE_SOURCES = ["ElectricalFiled.cu", "Bderivate.cu", "SplineGridConvIR2R.cu", "UpContinuation_gpu.cu",
                  "EFInterp2Rx.cu", "initialize_UpCont_gpu_resources.cu"]


def reference_present():
    return all(os.path.exists(os.path.join(REF, f)) for f in HOST_SOURCES + DEVICE_SOURCES + ["FTDT.h"])


def _cuda_home():
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def build_ref_host(verbose=False):
    if not reference_present():
        return None
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "ref_host")
    srcs = [os.path.join(REF, f) for f in HOST_SOURCES] + [os.path.join(HERE, "ref_host_driver.cpp")]
    if os.path.exists(exe) and all(os.path.getmtime(exe) > os.path.getmtime(s) for s in srcs):
        return exe
    cuda_inc = os.path.join(_cuda_home(), "include")
    # the C++ headers are pre-included because FTDT.h defines min/max macros
    cmd = ["g++", "-O0", "-fopenmp", "-w", "-Dpow10=exp10", "-include", "cmath", "-include", "limits",
           "-include", "algorithm", "-I", os.path.join(HERE, "shim"), "-I", REF,
           "-I", cuda_inc, "-o", exe] + srcs
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return exe


def build_ref_cpu_remap(verbose=False):
    """oracle/_ref/ref_cpu_remap: the reference's CPU spline remap (SplineGridConvIR2R_cpu.cpp,
    with its host setup files) under oracle/ref_cpu_remap_driver.cpp, for the CPU baseline."""
    if not reference_present() or not os.path.exists(os.path.join(REF, "SplineGridConvIR2R_cpu.cpp")):
        return None
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "ref_cpu_remap")
    srcs = [os.path.join(REF, f) for f in HOST_SOURCES + ["SplineGridConvIR2R_cpu.cpp"]] + \
        [os.path.join(HERE, "ref_cpu_remap_driver.cpp")]
    if os.path.exists(exe) and all(os.path.getmtime(exe) > os.path.getmtime(s) for s in srcs):
        return exe
    cuda_inc = os.path.join(_cuda_home(), "include")
    # optimised as the reference's Makefile compiles its C++ (-Ofast is -O3 with fast math there;
    # -O3 here, no -march=native so the binary is the same on every host of this architecture)
    cmd = ["g++", "-O3", "-fopenmp", "-w", "-Dpow10=exp10", "-include", "cmath", "-include", "limits",
           "-include", "vector", "-include", "algorithm", "-I", os.path.join(HERE, "shim"), "-I", REF,
           "-I", cuda_inc, "-o", exe] + srcs
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return exe


def cubin_path(src):
    return os.path.join(OUT, os.path.splitext(src)[0] + ".cubin")


def build_ref_cubins(verbose=False):
    """The reference's kernels as sm_103a device modules (the flags of its Makefile:56-60
    with the architecture replaced: no optimisation or fast-math options)."""
    if not reference_present():
        return None
    os.makedirs(OUT, exist_ok=True)
    nvcc = os.path.join(_cuda_home(), "bin", "nvcc")
    procs = []
    for s in DEVICE_SOURCES:
        src, out = os.path.join(REF, s), cubin_path(s)
        if os.path.exists(out) and os.path.getmtime(out) > os.path.getmtime(src):
            continue
        cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-w", "-DCUDA_DEVICE_ID=0",
               "-Dpow10=exp10", "-DdeviceOverlap=asyncEngineCount", "-I", os.path.join(HERE, "shim"), "-I", REF,
               src, "-o", out]
        if verbose:
            print(" ".join(cmd))
        procs.append((s, subprocess.Popen(cmd)))
    for s, p in procs:
        if p.wait() != 0:
            raise RuntimeError(f"nvcc failed on the reference's {s}")
    return OUT


if __name__ == "__main__":
    exe = build_ref_host(verbose=True)
    print(exe or "reference tree absent: nothing built")
    print(build_ref_cubins(verbose=True) or "")
    print(build_ref_cpu_remap(verbose=True) or "")
    sys.exit(0)
