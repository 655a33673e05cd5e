"""Build recipe for the reference-derived checkers under oracle/_ref/.

TEST INFRASTRUCTURE.  Compiles, from the reference source tree where it lies
(default /root/reference, override with TCSEM_REFERENCE_DIR), the reference's
host setup files together with oracle/ref_host_driver.cpp into
oracle/_ref/ref_host.  Nothing is copied out of the reference tree; only the
binary lands in oracle/_ref/ (git-ignored).  When the reference tree is absent
the build is skipped and the committed golden fixtures are used instead.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("TCSEM_REFERENCE_DIR", "/root/reference")
OUT = os.path.join(HERE, "_ref")

HOST_SOURCES = ["ModelingSetup.cpp", "SourceWave.cpp", "ModelGridMapping.cpp",
                "LoadRxTxPos.cpp", "logspace.cpp", "AuxiliaryMemory.cpp"]


def reference_present():
    return all(os.path.exists(os.path.join(REF, f)) for f in HOST_SOURCES + ["FTDT.h"])


def build_ref_host(verbose=False):
    if not reference_present():
        return None
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "ref_host")
    srcs = [os.path.join(REF, f) for f in HOST_SOURCES] + [os.path.join(HERE, "ref_host_driver.cpp")]
    if os.path.exists(exe) and all(os.path.getmtime(exe) > os.path.getmtime(s) for s in srcs):
        return exe
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    # -Dpow10=exp10: glibc dropped pow10; the shim directory supplies <fftw3.h>
    # the C++ headers are pre-included because FTDT.h defines min/max macros
    cmd = ["g++", "-O0", "-fopenmp", "-w", "-Dpow10=exp10", "-include", "cmath", "-include", "limits",
           "-include", "algorithm", "-I", os.path.join(HERE, "shim"), "-I", REF,
           "-I", cuda_inc, "-o", exe] + srcs
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return exe


if __name__ == "__main__":
    exe = build_ref_host(verbose=True)
    print(exe or "reference tree absent: nothing built")
    sys.exit(0)
