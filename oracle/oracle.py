"""ctypes binding of the FP64 CPU oracle (oracle/tcsem_oracle.c).

TEST INFRASTRUCTURE: imported by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py only.  The product library never loads it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libtcsem_oracle.so")
SRC = os.path.join(HERE, "tcsem_oracle.c")

FIELDS = {"Ex": 0, "Ey": 1, "Ez": 2, "Bx": 3, "By": 4, "Bz": 5, "BxAir": 6, "ByAir": 7, "Con": 8, "BzAir": 9}


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) > os.path.getmtime(SRC):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.run(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-Wall", "-Wno-format-truncation",
                    "-Wno-maybe-uninitialized", "-Wno-unused-result", "-o", tmp, SRC, "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        L.orc_open.restype = C.c_void_p
        L.orc_open.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_dims.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_params.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_get_darray.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_get_iarray.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_get_tx.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_field_size.restype = C.c_size_t
        L.orc_field_size.argtypes = [C.c_void_p, C.c_int]
        L.orc_get_field.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_set_field.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_zero_fields.argtypes = [C.c_void_p]
        L.orc_update_e.argtypes = [C.c_void_p, C.c_double, C.c_double]
        L.orc_add_source.argtypes = [C.c_void_p, C.c_int, C.c_double]
        L.orc_electric_field.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double]
        L.orc_bderivate.argtypes = [C.c_void_p, C.c_double]
        L.orc_spline_remap.argtypes = [C.c_void_p]
        L.orc_upcontinuation.argtypes = [C.c_void_p]
        L.orc_upcontinuation_padded.argtypes = [C.c_void_p]
        L.orc_rx_interp.restype = C.c_double
        L.orc_rx_interp.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.orc_run.restype = C.c_long
        L.orc_run.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_long]
        L.orc_schedule.restype = C.c_long
        L.orc_schedule.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_long]
        L.orc_set_dual_bipole_compat.argtypes = [C.c_void_p, C.c_int]
        L.orc_set_padded_plane.argtypes = [C.c_void_p, C.c_int]
        L.orc_num_threads.restype = C.c_int
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Oracle:
    """One loaded survey (all transmitters) held by the C oracle."""

    DNAMES = ["dx", "dy", "dz", "X", "Y", "Z", "Xn", "Yn", "dxk", "dyk", "dzk", "times", "tw", "dtw", "wave",
              "rx", "ry", "rz"]
    INAMES = ["xBzNew2old", "yBzNew2old", "xBzold2New", "yBzold2New", "xoldBx2NewBz", "yoldBy2NewBz",
              "rix", "riy", "riz"]

    def __init__(self, directory):
        err = C.create_string_buffer(256)
        h = lib().orc_open(directory.encode(), err, 256)
        if not h:
            raise RuntimeError(f"oracle: {err.value.decode()}")
        self.h = h
        d = np.zeros(16, dtype=np.int32)
        lib().orc_dims(h, _ptr(d))
        (self.L, self.M, self.N, self.L1, self.M1, self.AnLx_New, self.AnRx_New, self.Any_New, self.NRx, self.NTx,
         self.Nt, self.NComp, self.nefcmp, self.nsrc, self.IsLog, _) = [int(v) for v in d]
        p = np.zeros(8)
        lib().orc_params(h, _ptr(p))
        self.sfa1, self.sfa2, self.sita_t, self.minsita, self.mu0, self.mindx, self.T0, self.Tn = [float(v) for v in p]

    def close(self):
        if self.h:
            lib().orc_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def darray(self, name):
        n = {"dx": self.L, "dy": self.M, "dz": self.N, "X": self.L, "Y": self.M, "Z": self.N, "Xn": self.L1,
             "Yn": self.M1, "dxk": self.L, "dyk": self.M, "dzk": self.N, "times": self.Nt,
             "tw": 2 * self.nsrc + 1, "dtw": 2 * self.nsrc + 2, "wave": 2 * self.nsrc + 1,
             "rx": self.NRx, "ry": self.NRx, "rz": self.NRx}[name]
        out = np.zeros(n)
        lib().orc_get_darray(self.h, self.DNAMES.index(name), _ptr(out))
        return out

    def iarray(self, name):
        n = {"xBzNew2old": self.L1, "yBzNew2old": self.M1, "xBzold2New": self.L, "yBzold2New": self.M,
             "xoldBx2NewBz": self.L + 1, "yoldBy2NewBz": self.M + 1, "rix": self.NRx, "riy": self.NRx,
             "riz": self.NRx}[name]
        out = np.zeros(n, dtype=np.int32)
        lib().orc_get_iarray(self.h, self.INAMES.index(name), _ptr(out))
        return out

    def tx(self, t):
        iv = np.zeros(20, dtype=np.int32)
        dv = np.zeros(12)
        lib().orc_get_tx(self.h, t, _ptr(iv), _ptr(dv), None)
        rx = np.zeros(int(iv[1]), dtype=np.int32)
        lib().orc_get_tx(self.h, t, _ptr(iv), _ptr(dv), _ptr(rx))
        return iv, dv, rx

    def field_shape(self, name):
        L, M, N = self.L, self.M, self.N
        return {"Ex": (N + 1, M + 1, L), "Ey": (N + 1, M, L + 1), "Ez": (N, M + 1, L + 1), "Bx": (N, M, L + 1),
                "By": (N, M + 1, L), "Bz": (N + 1, M, L), "BxAir": (M, L + 1), "ByAir": (M + 1, L),
                "Con": (N, M, L), "BzAir": (self.M1, self.L1)}[name]

    def get(self, name):
        out = np.zeros(self.field_shape(name))
        lib().orc_get_field(self.h, FIELDS[name], _ptr(out))
        return out

    def set(self, name, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.shape == self.field_shape(name), (a.shape, self.field_shape(name))
        lib().orc_set_field(self.h, FIELDS[name], _ptr(a))

    def zero(self):
        lib().orc_zero_fields(self.h)

    def electric_field(self, itx, lam, dt, wave):
        lib().orc_electric_field(self.h, itx, lam, dt, wave)

    def update_e(self, lam, dt):
        lib().orc_update_e(self.h, lam, dt)

    def add_source(self, itx, wave):
        lib().orc_add_source(self.h, itx, wave)

    def bderivate(self, dt):
        lib().orc_bderivate(self.h, dt)

    def spline_remap(self):
        lib().orc_spline_remap(self.h)

    def upcontinuation(self):
        lib().orc_upcontinuation(self.h)

    def upcontinuation_padded(self):
        """The padded-plane variant of the continuation (not the reference's arithmetic), in the
        mode set by set_padded_plane (powers of two when unset)."""
        lib().orc_upcontinuation_padded(self.h)

    def rx_interp(self, comp, ir):
        return lib().orc_rx_interp(self.h, comp, ir)

    def set_dual_bipole_compat(self, on):
        lib().orc_set_dual_bipole_compat(self.h, int(bool(on)))

    def set_padded_plane(self, mode):
        """Whole runs continue the air field on the padded plane (orc_upcontinuation_padded):
        0 off, 1 powers of two, 2 lengths without prime factors above 5."""
        lib().orc_set_padded_plane(self.h, int(mode))

    def run(self, itx=0, max_steps=-1):
        iv, _, _ = self.tx(itx)
        out = np.zeros((int(iv[1]), self.NComp, self.Nt))
        n = lib().orc_run(self.h, itx, _ptr(out), max_steps)
        return out, int(n)

    def schedule(self, cap=1 << 20):
        n = lib().orc_schedule(self.h, None, None, None, None, 0)
        a = [np.zeros(n) for _ in range(4)]
        lib().orc_schedule(self.h, _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), _ptr(a[3]), n)
        return dict(dt1=a[0], dt2=a[1], lam=a[2], wave=a[3], nsteps=int(n))


def num_threads():
    return int(lib().orc_num_threads())
