"""Bounds-checked kernels (compute-sanitizer stands in for nothing here).

The library built with -DTCSEM_CHECK (tcsem_fdtd_gb300/build.py build_check,
csrc/check.cuh) tests every computed global index of the kernels against its
array and records a miss in the device error word, which any later call turns
into TCSEM_ERR_CUDA.  The same runs -- whole runs in both precisions and step
orders, several z-chunk layouts, the stage entry points and a batch under
both schedules (per-kernel graph and persistent kernel) -- go
through the normal and the checked library in separate processes: the checked
one must report no miss, and its outputs must equal the normal library's bit
for bit (the checks never change the arithmetic).
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import os, sys, json
import numpy as np
sys.path.insert(0, __ROOT__)
import tcsem_fdtd_gb300.api as api
api.LIB_PATH = __LIB__
from tcsem_fdtd_gb300 import Batch, Simulation, inputs
cases = json.loads(__CASES__)
out = {}
for name, d in cases.items():
    for prec in (64, 32):
        for z, serial in ((0, False), (1, False), (4, True), (5, False)):
            with Simulation(d, precision=prec, zchunks=z, serial_boundary=serial) as sim:
                out[f"{name}_{prec}_{z}_{int(serial)}"] = sim.run(0)
    with Simulation(d, precision=64, zchunks=3) as sim:  # the stage entry points on random fields
        rng = np.random.default_rng(3)
        for f in ("Ex", "Ey", "Ez", "Bx", "By", "Bz"):
            sim.set(f, rng.standard_normal(sim.field_shape(f)))
        sim.select_tx(0)
        sim.upcontinuation()
        sim.electric_field(1e-3, 1e-6, 0.5)
        sim.bderivate(1e-6)
        sim.fused_step(1e-3, 1e-6, 1e-6, 0.5)
        sim.synchronize()  # reads the device error word
        for f in ("Ex", "Ey", "Ez", "Bx", "By", "Bz", "BxAir", "ByAir"):
            out[f"{name}_stage_{f}"] = sim.get(f)
for tag, persistent in (("batch", False), ("persistent", True)):
    with Batch(precision=32, persistent=persistent) as b:
        slots = [b.add(d) for d in cases.values()]
        while b.stats()["running"]:
            b.advance(64)
        b.poll()
        for n, s in zip(cases, slots):
            out[f"{n}_{tag}"] = b.traces(s)
np.savez(__OUT__, **out)
"""


@pytest.fixture(scope="module")
def libs():
    from tcsem_fdtd_gb300 import build

    return build.build(), build.build_check()


def run_with(lib, cases, path):
    code = SCRIPT.replace("__ROOT__", repr(ROOT)).replace("__LIB__", repr(lib))
    code = code.replace("__CASES__", repr(json.dumps(cases))).replace("__OUT__", repr(str(path)))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    return np.load(path)


def test_bounds_checked_kernels_report_nothing_and_change_nothing(libs, case_dir, tmp_path):
    lib, lib_check = libs
    cases = {n: case_dir(n) for n in ("tiny", "small", "txvar")}
    plain = run_with(lib, cases, tmp_path / "plain.npz")
    checked = run_with(lib_check, cases, tmp_path / "checked.npz")
    assert sorted(plain.files) == sorted(checked.files)
    differ = [k for k in plain.files if not np.array_equal(plain[k], checked[k])]
    assert not differ, differ
