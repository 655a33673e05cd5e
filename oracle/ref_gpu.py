"""Receiver traces computed by the reference's own CUDA kernels.

TEST INFRASTRUCTURE.  oracle/ref_gpu_driver.cu is the host side of the
reference's time loop; the device side is the reference's kernels compiled
from its tree into oracle/_ref/*.cubin (oracle/build_ref.py).  The setup
arrays come from the reference's host code (tests/golden/ref_host_<case>.npz),
the conductivity from the survey's Cond.bin.  Used by
tests/golden/gen_ref_gpu_golden.py to make the golden traces; the product
never loads it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ref_gpu_driver.cu")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libref_gpu.so")
CUBINS = os.path.join(HERE, "_ref")


class Inputs(C.Structure):
    _fields_ = [("mp_i", C.c_int * 23), ("mp_d", C.c_double * 5)] + \
        [(n, C.c_void_p) for n in ("dx", "dy", "dz", "Z", "X", "Y", "Xn", "Yn")] + \
        [(n, C.c_void_p) for n in ("xBzNew2old", "yBzNew2old", "xBzold2New", "yBzold2New", "xoldBx2NewBz",
                                   "yoldBy2NewBz")] + \
        [("con", C.c_void_p), ("NRx", C.c_int)] + \
        [(n, C.c_void_p) for n in ("rx", "ry", "rz", "rix", "riy", "riz")] + \
        [("Nt", C.c_int), ("NComp", C.c_int), ("nefcmp", C.c_int), ("isComp", C.c_int * 6), ("times", C.c_void_p),
         ("nsrc", C.c_int), ("dtw", C.c_void_p), ("wave", C.c_void_p), ("sfa1", C.c_double), ("sfa2", C.c_double),
         ("minsita", C.c_double), ("miu", C.c_double), ("tx_i", C.c_int * 20), ("tx_d", C.c_double * 12),
         ("rxnum", C.c_void_p)]


def cubins_present():
    names = ["ElectricalFiled", "Bderivate", "SplineGridConvIR2R", "UpContinuation_gpu", "EFInterp2Rx",
             "initialize_UpCont_gpu_resources"]
    return all(os.path.exists(os.path.join(CUBINS, n + ".cubin")) for n in names)


def build():
    os.makedirs(BUILD, exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) > os.path.getmtime(SRC):
        return LIB
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.run([nvcc, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-o", tmp, SRC, "-lcuda", "-lcufft",
                    "-lcusparse"], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.refgpu_run.restype = C.c_int
        _lib.refgpu_run.argtypes = [C.c_char_p, C.POINTER(Inputs), C.c_void_p, C.c_long, C.POINTER(C.c_long),
                                    C.POINTER(C.c_double), C.c_char_p, C.c_int]
    return _lib


def run(case_dir, host_golden, itx=0, max_steps=-1):
    """Traces [nr][NComp][Nt] of transmitter `itx` (the first one is the only transmitter the
    reference defines), the steps taken and the device time of the step loop in ms."""
    g = {k: np.ascontiguousarray(v) for k, v in dict(np.load(host_golden)).items()}
    dims = g["dims"]
    L, M, N, L1, M1 = (int(v) for v in dims[:5])
    NRx, Nt, NComp, nefcmp, nsrc = int(dims[8]), int(dims[10]), int(dims[11]), int(dims[12]), int(dims[13])
    con = np.fromfile(os.path.join(case_dir, "Cond.bin"), dtype="<f8")
    assert con.size == L * M * N, (con.size, L, M, N)
    keep = [con]
    inp = Inputs()
    inp.mp_i[:] = [int(v) for v in g["mp_i"]]
    inp.mp_d[:] = [float(v) for v in g["mp_d"]]

    def p(a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        keep.append(a)
        return a.ctypes.data

    for n in ("dx", "dy", "dz", "Z", "X", "Y", "Xn", "Yn"):
        setattr(inp, n, p(g[n], np.float64))
    for n in ("xBzNew2old", "yBzNew2old", "xBzold2New", "yBzold2New", "xoldBx2NewBz", "yoldBy2NewBz"):
        setattr(inp, n, p(g[n], np.int32))
    inp.con = p(con, np.float64)
    inp.NRx = NRx
    for n in ("rx", "ry", "rz"):
        setattr(inp, n, p(g[n], np.float64))
    for n in ("rix", "riy", "riz"):
        setattr(inp, n, p(g[n], np.int32))
    inp.Nt, inp.NComp, inp.nefcmp = Nt, NComp, nefcmp
    inp.isComp[:] = [int(v) for v in g["isComp"]]
    inp.times = p(g["times"], np.float64)
    inp.nsrc = nsrc
    inp.dtw = p(g["dtw"], np.float64)
    inp.wave = p(g["wave"], np.float64)
    sfa1, sfa2, _sita_t, minsita, miu = (float(v) for v in g["params"][:5])
    inp.sfa1, inp.sfa2, inp.minsita, inp.miu = sfa1, sfa2, minsita, miu
    inp.tx_i[:] = [int(v) for v in g[f"tx{itx}_i"]]
    inp.tx_d[:] = [float(v) for v in g[f"tx{itx}_d"]]
    inp.rxnum = p(g[f"tx{itx}_rx"], np.int32)
    nr = int(g[f"tx{itx}_i"][1])
    out = np.zeros((nr, NComp, Nt))
    steps, ms = C.c_long(0), C.c_double(0)
    err = C.create_string_buffer(512)
    rc = lib().refgpu_run(CUBINS.encode(), C.byref(inp), out.ctypes.data, max_steps, C.byref(steps), C.byref(ms),
                          err, 512)
    if rc != 0:
        raise RuntimeError(f"reference kernels: {err.value.decode()}")
    return out, int(steps.value), float(ms.value)
