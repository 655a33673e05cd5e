"""Persistent batch schedule (tcsem_opts.persistent_batch): every block of graph_steps steps
of all slots is one cooperative launch whose CTAs take boundary, sweep and receiver items
from a device queue of the stages whose inputs are complete.

Within a slot the stages run in the order the per-kernel launches give them (boundary
rows, columns, inverse rows, bilinear remap, sweep of every z-chunk, receivers), on the
same per-CTA code and data, so each slot's traces must equal the graph-scheduled batch and
the survey run alone (1e-12 FP64 / 1e-6 FP32 of each trace's peak).  The schedule's wait
for a ready stage is bounded: the self-test makes it give up on a queue that nothing fills
and checks that the device stays usable.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {64: 1e-12, 32: 1e-6}


def rel_err(got, exp):
    peak = np.abs(exp).max(axis=2, keepdims=True)
    return float((np.abs(got - exp) / np.where(peak > 0, peak, 1.0)).max())


@pytest.fixture(scope="module")
def built():
    from tcsem_fdtd_gb300 import build

    build.build()
    return True


def alone(d, precision, itx=0, zchunks=1, top_planes=0):
    from tcsem_fdtd_gb300 import Simulation

    with Simulation(d, precision=precision, zchunks=zchunks, top_planes=top_planes) as sim:
        return sim.run(itx)


def run_to_end(b, block=64, limit=100000):
    done = set()
    for _ in range(limit):
        if b.stats()["running"] == 0:
            break
        b.advance(block)
        done.update(b.poll())
    return done


def batch_traces(dirs, precision, **kw):
    from tcsem_fdtd_gb300 import Batch

    with Batch(precision=precision, **kw) as b:
        slots = [b.add(d, itx) for d, itx in dirs]
        assert run_to_end(b) == set(slots)
        out = []
        for s in slots:
            info = b.info(s)
            assert info["steps_done"] == info["nsteps"]
            out.append((info, b.traces(s)))
        return out


@pytest.mark.parametrize("precision", [64, 32])
def test_persistent_batch_equals_graph_batch_and_alone(built, case_dir, precision):
    # a grid three sweep tiles wide with a partial last tile among surveys one tile wide
    cases = [("tiny", 0), ("small", 0), ("txvar", 3), ("halfspace_64x64x48", 0), ("wide_142x36x25", 0)]
    dirs = [(case_dir(n), itx) for n, itx in cases]
    per = batch_traces(dirs, precision, persistent=True)
    graph = batch_traces(dirs, precision)
    for (d, itx), (info, got), (_, ref) in zip(dirs, per, graph):
        assert info["launches_per_step"] == 0
        exp = alone(d, precision, itx)
        nr = exp.shape[0]
        assert np.all(np.isfinite(got[:nr]))
        assert rel_err(got[:nr], ref[:nr]) <= TOL[precision], (d, itx)
        assert rel_err(got[:nr], exp) <= TOL[precision], (d, itx)


def test_persistent_slots_join_and_leave_between_blocks(built, case_dir):
    """A survey that joins while others run, and one that leaves early: the remaining slots'
    traces equal each survey alone."""
    from tcsem_fdtd_gb300 import Batch

    d1, d2, d3 = case_dir("small"), case_dir("tiny"), case_dir("txvar")
    with Batch(precision=32, graph_steps=32, persistent=True) as b:
        s1 = b.add(d1)
        s3 = b.add(d3, 1)
        b.advance(96)
        s2 = b.add(d2)
        b.advance(64)
        b.remove(s3)
        done = run_to_end(b, block=32)
        assert {s1, s2} <= done
        for d, s in ((d1, s1), (d2, s2)):
            exp = alone(d, 32)
            assert rel_err(b.traces(s, nr=exp.shape[0]), exp) <= TOL[32]


@pytest.mark.parametrize("zchunks", [2, -1])
def test_persistent_batch_with_z_chunks(built, case_dir, zchunks):
    """Slots of several z-chunks (set, or chosen by the layout autotuner, which times the
    persistent blocks): the sweep stage covers every chunk, whose Bz prefix offsets carry
    across the chunks as in the per-kernel schedule."""
    dirs = [(case_dir("small"), 0), (case_dir("halfspace_64x64x48"), 0), (case_dir("wide_142x36x25"), 0)]
    for (d, itx), (info, got) in zip(dirs, batch_traces(dirs, 32, zchunks=zchunks, persistent=True)):
        if zchunks > 0:
            assert info["zchunks"] == zchunks
        top = info["top_planes"] if info["top_planes"] > 0 else -1
        exp = alone(d, 32, itx, zchunks=info["zchunks"], top_planes=top)
        assert rel_err(got[: exp.shape[0]], exp) <= TOL[32], (d, info["zchunks"], top)


def test_queue_wait_gives_up_and_the_device_stays_usable(built, case_dir):
    from tcsem_fdtd_gb300.api import selftest_queue_wait

    assert selftest_queue_wait(0, 20_000_000) == 1  # 20 ms
    assert selftest_queue_wait(0, 1) == 1
    d = case_dir("tiny")
    ((info, got),) = batch_traces([(d, 0)], 64, persistent=True)
    exp = alone(d, 64)
    assert rel_err(got[: exp.shape[0]], exp) <= TOL[64]
