"""Python mirror of the C ABI in include/tcsem.h (ctypes, no torch types).

The library is the in-tree ``libtcsem.so`` built by :mod:`tcsem_fdtd_gb300.build`.
There is no CPU path: if the library or a CUDA device is missing, opening a
simulation raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libtcsem.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "tcsem.h")

STATUS = {0: "OK", 1: "IO", 2: "PARSE", 3: "INVALID", 4: "CUDA", 5: "NOMEM", 6: "STATE", 7: "NUMERIC"}
COMP = {"Ex": 0, "Ey": 1, "Ez": 2, "Bx": 3, "By": 4, "Bz": 5, "BxAir": 6, "ByAir": 7, "Con": 8}


class TcsemError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"tcsem {STATUS.get(status, status)}: {msg}")
        self.status = status


class Opts(C.Structure):
    _fields_ = [("precision", C.c_int), ("device", C.c_int), ("fix_dual_bipole", C.c_int), ("graph_steps", C.c_int),
                ("zchunks", C.c_int), ("serial_boundary", C.c_int), ("top_planes", C.c_int),
                ("padded_plane", C.c_int), ("persistent_batch", C.c_int)]


class Info(C.Structure):
    _fields_ = [("L", C.c_int), ("M", C.c_int), ("N", C.c_int), ("L1", C.c_int), ("M1", C.c_int),
                ("NRx", C.c_int), ("NTx", C.c_int), ("Nt", C.c_int), ("NComp", C.c_int), ("nefcmp", C.c_int),
                ("nsteps", C.c_long), ("precision", C.c_int), ("device_bytes", C.c_size_t),
                ("launches_per_step", C.c_int), ("zchunks", C.c_int), ("top_planes", C.c_int),
                ("uploaded_bytes", C.c_size_t)]


# records of the in-memory open (tcsem_model / tcsem_transmitter / tcsem_survey)
MODEL_FIELDS = ["sfa1", "sfa2", "n1", "sita_t", "x0", "y0", "z0", "dxmin", "dymin", "dzmin", "arg1", "arg2",
                "ALx2", "ALx1", "Nx", "ARx1", "ARx2", "Ay2", "Ay1", "Ny", "Az2", "Az1", "Nz"]


class ModelRec(C.Structure):
    _fields_ = [(f, C.c_int if f in ("n1", "ALx2", "ALx1", "Nx", "ARx1", "ARx2", "Ay2", "Ay1", "Ny", "Az2", "Az1",
                                   "Nz") else C.c_double) for f in MODEL_FIELDS] + [("con", C.POINTER(C.c_double))]


class TxRec(C.Structure):
    _fields_ = [("ort", C.c_int)] + [(f, C.c_double) for f in ("len", "x", "y", "z", "azi", "dip", "len1", "x1",
                                                                 "y1", "z1", "azi1", "dip1")] + \
        [("nr", C.c_int), ("rx", C.POINTER(C.c_int))]


class SurveyRec(C.Structure):
    _fields_ = [("T0", C.c_double), ("Tn", C.c_double), ("Nt", C.c_int), ("IsLog", C.c_int), ("comps", C.c_int * 6),
                ("NRx", C.c_int), ("rx_xyz", C.POINTER(C.c_double)), ("NTx", C.c_int), ("tx", C.POINTER(TxRec))]


def declared_functions():
    """Names of the functions that include/tcsem.h declares."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tcsem_[a-z0-9_]+)\s*\(", text)))


_lib = None


def library():
    """Load libtcsem.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OSError(f"{LIB_PATH} is missing: build it with `python -m tcsem_fdtd_gb300.build`")
    L = C.CDLL(LIB_PATH)
    vp, dp, ip, i, d, l_ = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_int, C.c_double, C.c_long
    sig = {
        "tcsem_default_opts": (None, [C.POINTER(Opts)]),
        "tcsem_open_dir": (i, [C.c_char_p, C.POINTER(Opts), C.POINTER(vp)]),
        "tcsem_open": (i, [C.POINTER(ModelRec), C.POINTER(SurveyRec), C.POINTER(Opts), C.POINTER(vp)]),
        "tcsem_close": (i, [vp]),
        "tcsem_last_error": (C.c_char_p, [vp]),
        "tcsem_open_error": (C.c_char_p, []),
        "tcsem_get_info": (i, [vp, C.POINTER(Info)]),
        "tcsem_run": (i, [vp, i, dp]),
        "tcsem_write_bout": (i, [vp, i, dp, C.c_char_p]),
        "tcsem_begin": (i, [vp, i]),
        "tcsem_advance": (i, [vp, l_, ip]),
        "tcsem_get_traces": (i, [vp, dp]),
        "tcsem_synchronize": (i, [vp]),
        "tcsem_save_state": (i, [vp, C.c_char_p]),
        "tcsem_load_state": (i, [vp, C.c_char_p]),
        "tcsem_select_tx": (i, [vp, i]),
        "tcsem_upcontinuation": (i, [vp]),
        "tcsem_upcontinuation_noalloc": (i, [vp]),
        "tcsem_electric_field": (i, [vp, d, d, d]),
        "tcsem_bderivate": (i, [vp, d]),
        "tcsem_fused_step": (i, [vp, d, d, d, d]),
        "tcsem_rx_sample": (i, [vp, i, i, dp]),
        "tcsem_get_field": (i, [vp, i, dp]),
        "tcsem_set_field": (i, [vp, i, dp]),
        "tcsem_field_size": (i, [vp, i, C.POINTER(C.c_size_t)]),
        "tcsem_get_waveform": (i, [vp, ip, dp, dp, dp]),
        "tcsem_get_schedule": (i, [vp, dp, dp, dp, dp, l_]),
        "tcsem_time_steps": (i, [vp, i, l_, dp, dp, dp]),
        "tcsem_timed_advance": (i, [vp, l_, dp]),
        "tcsem_selftest_bounded_wait": (i, [i, i, ip]),
        "tcsem_selftest_queue_wait": (i, [i, C.c_longlong, ip]),
    }
    sig.update({
        "tcsem_batch_create": (i, [C.POINTER(Opts), C.c_size_t, C.POINTER(vp)]),
        "tcsem_batch_destroy": (i, [vp]),
        "tcsem_batch_error": (C.c_char_p, [vp]),
        "tcsem_batch_add": (i, [vp, C.c_char_p, i, ip]),
        "tcsem_batch_advance": (i, [vp, l_]),
        "tcsem_batch_poll": (i, [vp, ip, i, ip]),
        "tcsem_batch_slot_info": (i, [vp, i, C.POINTER(Info), C.POINTER(C.c_long)]),
        "tcsem_batch_traces": (i, [vp, i, dp]),
        "tcsem_batch_remove": (i, [vp, i]),
        "tcsem_batch_write_bout": (i, [vp, i, C.c_char_p]),
        "tcsem_batch_stats": (i, [vp, ip, ip, C.POINTER(C.c_size_t)]),
    })
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def selftest_bounded_wait(device=0, polls=1000):
    """tcsem_selftest_bounded_wait: 1 when a wait on an mbarrier that nothing completes gave up."""
    g = C.c_int(0)
    st = library().tcsem_selftest_bounded_wait(device, polls, C.byref(g))
    if st != 0:
        raise TcsemError(st, "bounded-wait self-test failed")
    return g.value


def selftest_queue_wait(device=0, wait_ns=20_000_000):
    """tcsem_selftest_queue_wait: 1 when the persistent batch kernel's wait for a stage that
    nothing publishes gave up after wait_ns."""
    g = C.c_int(0)
    st = library().tcsem_selftest_queue_wait(device, int(wait_ns), C.byref(g))
    if st != 0:
        raise TcsemError(st, "queue-wait self-test failed")
    return g.value


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def memory_records(model, survey):
    """tcsem_model / tcsem_survey records for tcsem_open from plain values.

    model:  the FDTD_setup.in fields of MODEL_FIELDS plus ``con`` (conductivity [N][M][L]);
    survey: ``T0 Tn Nt IsLog comps`` (Receiver.in), ``rx_xyz`` ([NRx][3]) and ``tx``, a list of
            dicts with ``ort len x y z`` (+ ``azi dip`` in degrees for ort 4/5, + ``len1 x1 y1 z1
            azi1 dip1`` for ort 5) and ``rx`` (1-based receiver ids).
    Returns (model record, survey record, arrays the records point into)."""
    keep = []
    m = ModelRec()
    for f in MODEL_FIELDS:
        setattr(m, f, model[f])
    con = np.ascontiguousarray(model["con"], dtype=np.float64)
    keep.append(con)
    m.con = _dptr(con)
    s = SurveyRec()
    s.T0, s.Tn, s.Nt, s.IsLog = survey["T0"], survey["Tn"], survey["Nt"], survey["IsLog"]
    s.comps[:] = [int(v) for v in survey["comps"]]
    xyz = np.ascontiguousarray(survey["rx_xyz"], dtype=np.float64).reshape(-1, 3)
    keep.append(xyz)
    s.NRx, s.rx_xyz = xyz.shape[0], _dptr(xyz)
    txs = (TxRec * len(survey["tx"]))()
    for q, t in enumerate(survey["tx"]):
        r = txs[q]
        r.ort = int(t["ort"])
        for f in ("len", "x", "y", "z", "azi", "dip", "len1", "x1", "y1", "z1", "azi1", "dip1"):
            setattr(r, f, float(t.get(f, 0.0)))
        ids = np.ascontiguousarray(t["rx"], dtype=np.int32)
        keep.append(ids)
        r.nr, r.rx = len(ids), ids.ctypes.data_as(C.POINTER(C.c_int))
    keep.append(txs)
    s.NTx, s.tx = len(survey["tx"]), txs
    return m, s, keep


class Simulation:
    """One survey on one GPU: the handle of include/tcsem.h.

    Opened from a survey directory (tcsem_open_dir), or with ``model=`` and ``survey=`` from
    host values (tcsem_open, see :func:`memory_records`)."""

    def __init__(self, directory=None, precision=32, device=0, fix_dual_bipole=False, graph_steps=0, zchunks=0,
                 serial_boundary=False, top_planes=0, padded_plane=False, model=None, survey=None):
        L = library()
        o = Opts()
        L.tcsem_default_opts(C.byref(o))
        o.precision, o.device, o.fix_dual_bipole, o.graph_steps = precision, device, int(fix_dual_bipole), graph_steps
        o.zchunks = zchunks
        o.serial_boundary = int(serial_boundary)
        o.top_planes = top_planes
        o.padded_plane = int(padded_plane)  # 0, 1 (powers of two) or 2 (5-smooth lengths)
        h = C.c_void_p()
        if directory is not None:
            st = L.tcsem_open_dir(os.fsencode(directory), C.byref(o), C.byref(h))
        else:
            mrec, srec, _keep = memory_records(model, survey)
            st = L.tcsem_open(C.byref(mrec), C.byref(srec), C.byref(o), C.byref(h))
        if st != 0:
            raise TcsemError(st, L.tcsem_open_error().decode())
        self._h = h
        inf = Info()
        L.tcsem_get_info(h, C.byref(inf))
        self.info = {f: getattr(inf, f) for f, _ in Info._fields_}
        self.precision = precision

    # ------------------------------------------------------------------ plumbing
    def _check(self, st):
        if st != 0:
            raise TcsemError(st, library().tcsem_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            library().tcsem_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --------------------------------------------------------------- whole runs
    def run(self, itx=0, nr=None):
        """All steps of transmitter itx; returns traces [nr][NComp][Nt]."""
        i = self.info
        buf = np.zeros(i["NRx"] * i["NComp"] * i["Nt"])
        self._check(library().tcsem_run(self._h, itx, _dptr(buf)))
        n = nr if nr is not None else i["NRx"]
        return buf[: n * i["NComp"] * i["Nt"]].reshape(n, i["NComp"], i["Nt"])

    def write_bout(self, itx, traces, path):
        t = np.ascontiguousarray(traces, dtype=np.float64)
        self._check(library().tcsem_write_bout(self._h, itx, _dptr(t), os.fsencode(path)))

    def begin(self, itx=0):
        self._check(library().tcsem_begin(self._h, itx))

    def advance(self, nsteps):
        done = C.c_int(0)
        self._check(library().tcsem_advance(self._h, nsteps, C.byref(done)))
        return bool(done.value)

    def traces(self, nr):
        i = self.info
        buf = np.zeros(i["NRx"] * i["NComp"] * i["Nt"])
        self._check(library().tcsem_get_traces(self._h, _dptr(buf)))
        return buf[: nr * i["NComp"] * i["Nt"]].reshape(nr, i["NComp"], i["Nt"])

    def synchronize(self):
        self._check(library().tcsem_synchronize(self._h))

    def save_state(self, path):
        """tcsem_save_state: checkpoint of the run in progress."""
        self._check(library().tcsem_save_state(self._h, os.fsencode(path)))

    def load_state(self, path):
        """tcsem_load_state: continue a saved run (same survey, precision and z-chunk layout)."""
        self._check(library().tcsem_load_state(self._h, os.fsencode(path)))

    # -------------------------------------------------------------- stage seam
    def select_tx(self, itx):
        self._check(library().tcsem_select_tx(self._h, itx))

    def upcontinuation(self):
        self._check(library().tcsem_upcontinuation(self._h))

    def upcontinuation_noalloc(self):
        """The boundary step with the library's static scratch (allocates nothing)."""
        self._check(library().tcsem_upcontinuation_noalloc(self._h))

    def electric_field(self, lam, dt, wave):
        self._check(library().tcsem_electric_field(self._h, lam, dt, wave))

    def bderivate(self, dt):
        self._check(library().tcsem_bderivate(self._h, dt))

    def fused_step(self, lam, dt, dtb, wave):
        self._check(library().tcsem_fused_step(self._h, lam, dt, dtb, wave))

    def rx_sample(self, efield, slot, nr):
        out = np.zeros(self.info["NComp"] * self.info["NRx"])
        self._check(library().tcsem_rx_sample(self._h, int(bool(efield)), slot, _dptr(out)))
        return out[: self.info["NComp"] * nr].reshape(self.info["NComp"], nr)

    # ------------------------------------------------------------ field access
    def field_shape(self, name):
        L, M, N = self.info["L"], self.info["M"], self.info["N"]
        return {"Ex": (N + 1, M + 1, L), "Ey": (N + 1, M, L + 1), "Ez": (N, M + 1, L + 1), "Bx": (N, M, L + 1),
                "By": (N, M + 1, L), "Bz": (N + 1, M, L), "BxAir": (M, L + 1), "ByAir": (M + 1, L),
                "Con": (N, M, L)}[name]

    def get(self, name):
        out = np.zeros(self.field_shape(name))
        self._check(library().tcsem_get_field(self._h, COMP[name], _dptr(out)))
        return out

    def set(self, name, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.shape == self.field_shape(name)
        self._check(library().tcsem_set_field(self._h, COMP[name], _dptr(a)))

    def waveform(self):
        n = C.c_int(0)
        self._check(library().tcsem_get_waveform(self._h, C.byref(n), None, None, None))
        t, dt, w = (np.zeros(2 * n.value + 1) for _ in range(3))
        self._check(library().tcsem_get_waveform(self._h, C.byref(n), _dptr(t), _dptr(dt), _dptr(w)))
        return t, dt, w

    def schedule(self):
        n = self.info["nsteps"]
        a = [np.zeros(n) for _ in range(4)]
        self._check(library().tcsem_get_schedule(self._h, *[_dptr(x) for x in a], n))
        return dict(dt1=a[0], dt2=a[1], lam=a[2], wave=a[3], nsteps=n)

    def timed_advance(self, nsteps):
        """Advance `nsteps` steps; returns their device time in ms (CUDA events on the handle's stream)."""
        ms = C.c_double()
        self._check(library().tcsem_timed_advance(self._h, nsteps, C.byref(ms)))
        return ms.value

    def time_steps(self, itx, nsteps):
        """Device time (ms) of `nsteps` captured steps, and of one sweep / one boundary pass."""
        tot, sw, bn = C.c_double(), C.c_double(), C.c_double()
        self._check(library().tcsem_time_steps(self._h, itx, nsteps, C.byref(tot), C.byref(sw), C.byref(bn)))
        return tot.value, sw.value, bn.value


class Batch:
    """Many surveys advanced together (tcsem_batch_* of include/tcsem.h)."""

    def __init__(self, precision=32, device=0, budget=0, graph_steps=0, zchunks=0, top_planes=0, padded_plane=False,
                 persistent=False):
        L = library()
        o = Opts()
        L.tcsem_default_opts(C.byref(o))
        o.precision, o.device, o.graph_steps, o.zchunks = precision, device, graph_steps, zchunks
        o.top_planes = top_planes
        o.padded_plane = int(padded_plane)
        o.persistent_batch = int(persistent)
        h = C.c_void_p()
        st = L.tcsem_batch_create(C.byref(o), int(budget), C.byref(h))
        if st != 0:
            raise TcsemError(st, L.tcsem_batch_error(None).decode())
        self._h = h

    def _check(self, st):
        if st != 0:
            raise TcsemError(st, library().tcsem_batch_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            library().tcsem_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, directory, itx=0):
        """Set up one survey as a new slot; raises TcsemError (status 5) when it does not fit."""
        slot = C.c_int()
        self._check(library().tcsem_batch_add(self._h, os.fsencode(directory), itx, C.byref(slot)))
        return slot.value

    def advance(self, nsteps):
        self._check(library().tcsem_batch_advance(self._h, nsteps))

    def poll(self):
        """Slots whose runs are complete (waits for the enqueued work)."""
        n = C.c_int()
        self._check(library().tcsem_batch_poll(self._h, None, 0, C.byref(n)))
        ids = (C.c_int * max(1, n.value))()
        self._check(library().tcsem_batch_poll(self._h, ids, n.value, C.byref(n)))
        return list(ids[: n.value])

    def info(self, slot):
        inf, done = Info(), C.c_long()
        self._check(library().tcsem_batch_slot_info(self._h, slot, C.byref(inf), C.byref(done)))
        d = {f: getattr(inf, f) for f, _ in Info._fields_}
        d["steps_done"] = done.value
        return d

    def traces(self, slot, nr=None):
        i = self.info(slot)
        buf = np.zeros(i["NRx"] * i["NComp"] * i["Nt"])
        self._check(library().tcsem_batch_traces(self._h, slot, _dptr(buf)))
        n = nr if nr is not None else i["NRx"]
        return buf[: n * i["NComp"] * i["Nt"]].reshape(n, i["NComp"], i["Nt"])

    def write_bout(self, slot, path):
        self._check(library().tcsem_batch_write_bout(self._h, slot, os.fsencode(path)))

    def remove(self, slot):
        self._check(library().tcsem_batch_remove(self._h, slot))

    def stats(self):
        n, r, b = C.c_int(), C.c_int(), C.c_size_t()
        self._check(library().tcsem_batch_stats(self._h, C.byref(n), C.byref(r), C.byref(b)))
        return {"slots": n.value, "running": r.value, "device_bytes": b.value}
