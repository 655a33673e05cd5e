"""The CUDA path against receiver traces computed by the reference's own CUDA kernels
(tests/golden/ref_gpu_<case>.npz; tests/test_oracle_reference_kernels.py says how they were
made and checks the oracle against them).

Whole runs, default layout, on tiny, small, every transmitter orientation (txvar), the
three-tile grid, the 1 S/m half-space survey (64 x 64 x 48), the 1-D marine survey
(128 x 128 x 96) and the 3-D marine survey at 256 x 256 x 160 with 35-cell boundary strips.
(With the 40-cell strips of marine3d_256x256x160 the reference's own run is not finite:
tests/test_oracle_reference_kernels.py.)  Criteria (tests/traces.py):

* FP64 build: 1e-8 of each signal trace's peak -- the survey's criterion for this
  comparison is 1e-4 above a noise floor at 1e-6 of the trace peak;
* FP32 production: 1 %; the measured error per survey is printed.
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

sys.path.insert(0, GOLDEN)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from traces import check_fp32, check_fp64, field_error  # noqa: E402

CASES = ["tiny", "small", "txvar", "wide_142x36x25", "halfspace_64x64x48", "marine1d_128x128x96"]


@pytest.fixture(scope="module")
def built():
    from tcsem_fdtd_gb300 import build

    build.build()
    return True


def reference(case, case_dir):
    import gen_oracle_traces as g

    z = np.load(os.path.join(GOLDEN, f"ref_gpu_{case}.npz"))
    d = case_dir(case)
    if not g.same_inputs(g.inputs_fingerprint(d), g.fingerprint_of(z)):
        pytest.fail(f"{case}: the seeded inputs differ from those of the reference run")
    return z, d


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("case", CASES)
def test_traces_match_the_reference_kernels(built, case_dir, case, precision):
    from tcsem_fdtd_gb300 import Simulation

    z, d = reference(case, case_dir)
    txs = sorted(int(k[2:-7]) for k in z.files if k.endswith("_traces"))
    with Simulation(d, precision=precision) as sim:
        for t in txs:
            exp = z[f"tx{t}_traces"]
            assert np.isfinite(exp).all()
            got = sim.run(t, nr=exp.shape[0])
            assert sim.info["nsteps"] == int(z[f"tx{t}_steps"])
            if precision == 64:
                err = check_fp64(got, exp, sim.info["nefcmp"])
            else:
                err = check_fp32(got, exp, sim.info["nefcmp"])
            print(f"{case} tx{t + 1} fp{precision} against the reference kernels: {err}")


@pytest.mark.parametrize("precision", [64, 32])
def test_traces_on_the_256_grid_match_the_reference_kernels(built, case_dir, precision):
    """marine3d_strip35_256x256x160, all 6884 steps.  The reference's own runs on this grid
    differ from each other by about 1e-9 of the largest trace (its kernels race on shared
    memory, tests/test_oracle_reference_kernels.py), which is up to 1e-3 of the weakest far
    receivers' peaks; the comparison is therefore on the survey's amplitude scale: 1e-7 of
    the largest trace of each field in FP64 (and the FP32 criterion of tests/traces.py)."""
    from tcsem_fdtd_gb300 import Simulation

    case = "marine3d_strip35_256x256x160"
    z, d = reference(case, case_dir)
    exp = z["tx0_traces"]
    with Simulation(d, precision=precision) as sim:
        got = sim.run(0)
        assert sim.info["nsteps"] == int(z["tx0_steps"])
        nefcmp = sim.info["nefcmp"]
    err = field_error(got, exp, nefcmp)
    print(f"{case} fp{precision} against the reference kernels: {err:.3e} of the largest trace")
    if precision == 64:
        assert err < 1e-7
    else:
        print(check_fp32(got, exp, nefcmp))
