"""Failure detection without a GPU fault.

* The bounded waits: a kernel waits on an mbarrier that nothing completes, gives
  up after a short poll limit and reports it through the device error word; the
  device stays usable (a survey then runs and matches the FP64 oracle).
* A survey whose conductivity holds a NaN: its traces are refused with
  TCSEM_ERR_NUMERIC, alone or as one slot of a batch, and the other slots of the
  batch still match their runs alone.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NUMERIC = 7  # TCSEM_ERR_NUMERIC


@pytest.fixture(scope="module")
def built():
    from oracle import oracle as orc
    from tcsem_fdtd_gb300 import build

    build.build()
    orc.build()
    return True


def nan_case(case_dir, tmp_path):
    """The tiny survey with one NaN conductivity cell in the middle of the grid."""
    import shutil

    src = case_dir("tiny")
    d = tmp_path / "tiny_nan"
    shutil.copytree(src, d)
    sig = np.fromfile(d / "Cond.bin", dtype="<f8")
    sig[sig.size // 2] = np.nan
    sig.tofile(d / "Cond.bin")
    return str(d)


def test_bounded_wait_gives_up_and_the_device_stays_usable(built, case_dir):
    from oracle.oracle import Oracle
    from tcsem_fdtd_gb300 import Simulation
    from tcsem_fdtd_gb300.api import selftest_bounded_wait

    assert selftest_bounded_wait(0, 1000) == 1
    assert selftest_bounded_wait(0, 1) == 1
    d = case_dir("tiny")
    exp, _ = Oracle(d).run(0)
    with Simulation(d, precision=64) as sim:
        got = sim.run(0, nr=exp.shape[0])
    assert np.abs(got - exp).max() <= 1e-8 * np.abs(exp).max()


def test_nan_conductivity_is_refused_at_the_traces(built, case_dir, tmp_path):
    from tcsem_fdtd_gb300 import Simulation, TcsemError

    with Simulation(nan_case(case_dir, tmp_path), precision=32) as sim:
        with pytest.raises(TcsemError) as e:
            sim.run(0)
        assert e.value.status == NUMERIC


def test_nan_slot_fails_alone_in_a_batch(built, case_dir, tmp_path):
    from tcsem_fdtd_gb300 import Batch, Simulation, TcsemError

    good = case_dir("small")
    with Simulation(good, precision=32, zchunks=1) as sim:
        exp = sim.run(0)
    with Batch(precision=32) as b:
        s_good = b.add(good)
        s_bad = b.add(nan_case(case_dir, tmp_path))
        while b.stats()["running"]:
            b.advance(64)
        b.poll()
        with pytest.raises(TcsemError) as e:
            b.traces(s_bad)
        assert e.value.status == NUMERIC
        got = b.traces(s_good)
    peak = np.abs(exp).max(axis=2, keepdims=True)
    assert float((np.abs(got - exp) / np.where(peak > 0, peak, 1.0)).max()) < 1e-6
    assert os.path.exists(good)
