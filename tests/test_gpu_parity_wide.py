"""The production sweep against the FP64 oracle on grids wider than one sweep tile and on
the survey configurations, with the default z-chunk layout and the overlapped step.

The fused sweep works on tiles of 64 x 8 cells: a tile recomputes the +x halo column and
the +y halo row it needs, and reads its x-neighbours' cells from its own TMA box.  The
grids here exercise those paths:

* wide_142x36x25: three x-tiles (the last one 14 cells wide) and five tile rows (the last
  one 4 rows high); transmitters cross the tile boundaries at i = 64, j = 16 and i = 128;
* halfspace_64x64x48 (the 1 S/m half-space survey), a whole run;
* marine1d_128x128x96, marine3d_256x256x160 and its variant with 35-cell boundary strips,
  the first 400 steps (the source window and the first samples) -- marine3d_256x256x160
  runs in the production layout of the bench: a one-plane top z-chunk beside the boundary,
  two lower chunks, the receiver kernel on its own stream.

The oracle takes minutes on the three survey grids, so their traces are stored in
tests/golden/oracle_traces_<case>.npz (tests/golden/gen_oracle_traces.py); a fingerprint
of the inputs is stored beside them and a test whose regenerated inputs differ computes the
oracle instead.

Tolerances (tests/traces.py): FP64 build 1e-8, FP32 production 1 %, of each trace's peak
for the traces that carry a signal and of the field's largest trace for the components that
vanish by symmetry.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from traces import check_fp32, check_fp64  # noqa: E402

STAGE_TOL = {64: 1e-10, 32: 2e-5}


def rel(a, b):
    s = np.abs(b).max()
    return float(np.abs(a - b).max() / s) if s > 0 else float(np.abs(a).max())


def trace_error(got, exp):
    """max over traces of max|got - exp| / max|exp| (traces with zero peak skipped)."""
    worst = 0.0
    for r in range(exp.shape[0]):
        for c in range(exp.shape[1]):
            pk = np.abs(exp[r, c]).max()
            if pk > 0:
                worst = max(worst, float(np.abs(got[r, c] - exp[r, c]).max() / pk))
    return worst


@pytest.fixture(scope="module")
def built():
    from tcsem_fdtd_gb300 import build
    from oracle import oracle as orc

    build.build()
    orc.build()
    return True


def oracle_traces(case_dir, case):
    """Stored oracle traces of `case` when the inputs match, else the oracle run now."""
    import gen_oracle_traces as g

    d = case_dir(case)
    tr, n, max_steps, fp = g.load(case)
    if g.same_inputs(g.inputs_fingerprint(d), fp):
        return d, tr, n, max_steps
    from oracle.oracle import Oracle

    orc = Oracle(d)
    tr, n = orc.run(0, max_steps=max_steps)
    return d, tr, n, max_steps


def run_product(d, precision, max_steps, **kw):
    """Traces of transmitter 1 after `max_steps` steps (all steps when negative)."""
    from tcsem_fdtd_gb300 import Simulation

    with Simulation(d, precision=precision, **kw) as sim:
        nr = sim.info["NRx"]
        if max_steps < 0:
            return sim.run(0), sim.info
        sim.begin(0)
        sim.advance(max_steps)
        return sim.traces(nr), sim.info


# ----------------------------------------------------------------- multi-tile grid


@pytest.mark.parametrize("zchunks", [0, 3])
@pytest.mark.parametrize("precision", [64, 32])
def test_fused_step_stage_on_three_x_tiles(built, case_dir, precision, zchunks):
    """One fused step from random fields on the 142 x 36 x 25 grid, with the source on and
    off, against E then B of the oracle -- every tile edge of the sweep in play."""
    from oracle.oracle import Oracle
    from tcsem_fdtd_gb300 import Simulation

    d = case_dir("wide_142x36x25")
    orc = Oracle(d)
    sched = orc.schedule()
    with Simulation(d, precision=precision, zchunks=zchunks) as sim:
        for itx in range(orc.NTx):
            for step in (4, 260):
                rng = np.random.default_rng(1000 * itx + step)
                for n in ("Ex", "Ey", "Ez", "Bx", "By", "Bz", "BxAir", "ByAir"):
                    a = rng.standard_normal(orc.field_shape(n))
                    orc.set(n, a)
                    sim.set(n, a)
                lam, dt, wave = sched["lam"][step], sched["dt1"][step], sched["wave"][step]
                dtb = 0.5 * (sched["dt1"][step] + sched["dt2"][step])
                sim.select_tx(itx)
                sim.fused_step(lam, dt, dtb, wave)
                orc.electric_field(itx, lam, dt, wave)
                orc.bderivate(dtb)
                for n in ("Ex", "Ey", "Ez", "Bx", "By", "Bz"):
                    assert rel(sim.get(n), orc.get(n)) < STAGE_TOL[precision], (itx, step, n)


@pytest.mark.parametrize("serial", [False, True])
@pytest.mark.parametrize("precision", [64, 32])
def test_whole_runs_on_three_x_tiles(built, case_dir, precision, serial):
    """Every transmitter of the 142 x 36 x 25 survey, default layout, overlapped (and
    serial) step order, against whole oracle runs."""
    from oracle.oracle import Oracle
    from tcsem_fdtd_gb300 import Simulation

    d = case_dir("wide_142x36x25")
    orc = Oracle(d)
    with Simulation(d, precision=precision, serial_boundary=serial) as sim:
        assert sim.info["zchunks"] >= 2
        for itx in range(orc.NTx):
            exp, n = orc.run(itx)
            got = sim.run(itx, nr=exp.shape[0])
            err = trace_error(got, exp)
            print(f"wide fp{precision} serial={serial} tx{itx + 1}: {n} steps, trace error {err:.3e}")
            assert err < (1e-8 if precision == 64 else 1e-2), (itx, err)


# ------------------------------------------------------------ survey configurations


@pytest.mark.parametrize("precision", [64, 32])
def test_halfspace_survey_whole_run(built, case_dir, precision):
    """The 1 S/m half-space survey (64 x 64 x 48, 3026 steps) in the default layout."""
    d, exp, n, _ = oracle_traces(case_dir, "halfspace_64x64x48")
    got, info = run_product(d, precision, -1)
    assert info["nsteps"] == n
    if precision == 64:
        err = check_fp64(got, exp, info["nefcmp"])
    else:
        err = check_fp32(got, exp, info["nefcmp"])
    print(f"halfspace_64x64x48 fp{precision}: {err}")


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("case", ["marine1d_128x128x96", "marine3d_256x256x160", "marine3d_strip35_256x256x160"])
def test_marine_surveys_first_400_steps(built, case_dir, case, precision):
    """The first 400 steps of the marine surveys in the production layout."""
    d, exp, n, max_steps = oracle_traces(case_dir, case)
    assert n == max_steps == 400
    got, info = run_product(d, precision, max_steps)
    if case == "marine3d_256x256x160" and precision == 32:
        assert info["zchunks"] == 3 and info["top_planes"] == 1 and info["launches_per_step"] == 7
    reached = np.nonzero(np.abs(exp).max(axis=(0, 1)))[0]
    assert len(reached) >= 10  # the window reaches the first samples
    # samples the oracle had not reached are still zero in the product too
    assert not np.abs(got[..., reached[-1] + 1:]).any()
    if precision == 64:
        err = check_fp64(got, exp, info["nefcmp"])
    else:
        err = check_fp32(got, exp, info["nefcmp"])
    print(f"{case} fp{precision}: {len(reached)} samples, {err}")
