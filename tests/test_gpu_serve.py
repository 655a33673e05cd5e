"""Serving loop: requests arriving over time share the device batch.

Every request's traces must be the same served in the mix as run alone
(same z-chunk layout: one chunk): within 1e-6 relative to each trace's peak (FP32).  A
budget that fits only part of the stream makes later requests wait for
earlier ones to leave; they still complete with the same results.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_err(got, exp):
    peak = np.abs(exp).max(axis=2, keepdims=True)
    return float((np.abs(got - exp) / np.where(peak > 0, peak, 1.0)).max())


@pytest.fixture(scope="module")
def built():
    from tcsem_fdtd_gb300 import build

    build.build()
    return True


def alone(d, itx=0):
    from tcsem_fdtd_gb300 import Simulation

    with Simulation(d, precision=32, zchunks=1) as sim:
        return sim.run(itx)


def stream(case_dir):
    from tcsem_fdtd_gb300.serve import Request

    names = [("small", 0), ("tiny", 0), ("txvar", 2), ("halfspace_64x64x48", 0), ("tiny", 0), ("txvar", 4)]
    return [Request(r, case_dir(n), 0.02 * r, itx) for r, (n, itx) in enumerate(names)]


@pytest.mark.parametrize("budget", [64 << 30, 0])
def test_served_results_equal_alone(built, case_dir, budget):
    from tcsem_fdtd_gb300.serve import Server, serve, summary

    reqs = stream(case_dir)
    if budget == 0:  # room for about two requests at a time, so later arrivals queue
        from tcsem_fdtd_gb300.api import Batch

        with Batch(precision=32) as b:
            biggest = max(b.info(b.add(r.directory, r.itx))["device_bytes"] for r in reqs)
        budget = 2 * biggest + (12 << 20)  # admission uses an estimate a few MB above the allocation
    srv = Server(budget=budget, block=32)
    try:
        wall = serve(reqs, srv)
    finally:
        srv.close()
    s = summary(reqs, wall)
    assert s["requests"] == len(reqs) and s["p99_latency_s"] >= s["p50_latency_s"] > 0
    for r in reqs:
        assert r.completed >= r.admitted >= r.arrival
        exp = alone(r.directory, r.itx)
        assert rel_err(r.traces[: exp.shape[0]], exp) <= 1e-6, r.directory
