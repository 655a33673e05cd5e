"""The oracle against the reference's own CUDA kernels.

tests/golden/ref_gpu_<case>.npz hold receiver traces that the reference's device code
computed on a GB300 (tests/golden/gen_ref_gpu_golden.py: the reference's kernels compiled
from its tree, FP64, driven in the order of its time loop with the setup arrays of its own
host code).  The oracle's restatement of the device half -- E and B updates, source
injection, spline remap, FFT continuation, bilinear remap, receiver interpolation and the
sampling state machine -- reproduces them (criteria of tests/traces.py, 1e-10 here):

* whole runs of tiny, small, every transmitter orientation (txvar, ort 1-5, the second
  bipole of ort 5 at the first bipole's cells as the reference does) and the three-tile
  grid wide_142x36x25 (measured 2.1e-11);
* the 1 S/m half-space survey, 3026 steps: the stored oracle run (measured 4.6e-9, 2e-8 here);
* the marine surveys: the first 400 steps the oracle ran against the samples the
  reference's whole run took in that window.

The reference defines only its first transmitter (its counters carry over); the other
transmitters of txvar and wide_142x36x25 ran with the reference's kernels from a zero state.

On the 256 x 256 x 160 grid the reference's kernels are not deterministic: repeated runs of
the same survey differ from each other, by up to 1.7e-9 of the largest trace after 800
steps (three runs of marine3d_strip35_256x256x160 on a GB300); on the smaller grids they
agree to 4e-15.  Its E and B kernels stage a plane of their inputs in shared memory and
refill it for the next plane without a barrier after the reads of the previous plane
(UpdateBx, Bderivate.cu:94-125; UpdateBy; UpdateEy/UpdateEz, ElectricalFiled.cu:178-345):
a warp that runs ahead overwrites values a neighbouring warp of the block has not read yet.
The oracle and the product compute each plane from its own values, and are compared with
that run on the scale of the survey's largest trace.

One reference run is not finite: marine3d_256x256x160, whose 40-cell boundary strips give
280 uniform continuation points per strip.  The reference's strip kernels
(Intep_BzIR2R_0x/1x/0y/1y, SplineGridConvIR2R.cu:180-498) run 256 threads per block over a
strip's points and stage the strip's spline nodes in shared memory with the block's own
threads (`if (threadIdx.x < n1)` inside `if (ix < AnLx_New ...)`): in the last block only
AnLx_New mod 256 threads are alive, so when that is smaller than the n1 = ALx1 + ALx2 + 4
nodes, the nodes above it are read from shared memory nobody wrote in that block.  On
marine3d_256x256x160 that is 280 mod 256 = 24 < 44, and every trace is NaN.  The oracle and
the product use the nodes the spline is defined on; the same grid with 35-cell strips
(187 points, one block) is pinned instead.
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, GOLDEN)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from traces import compare, field_error  # noqa: E402


def ref(case):
    return np.load(os.path.join(GOLDEN, f"ref_gpu_{case}.npz"))


def check(got, exp, nefcmp, tol):
    sig, res, per = compare(got, exp, nefcmp, 1e-6)
    assert sig < tol and res < tol, (sig, res, per)


@pytest.mark.parametrize("case", ["tiny", "small", "txvar", "wide_142x36x25"])
def test_oracle_whole_runs_match_the_reference_kernels(case, case_dir):
    import gen_oracle_traces as g
    from oracle.oracle import Oracle

    z = ref(case)
    d = case_dir(case)
    assert g.same_inputs(g.inputs_fingerprint(d), g.fingerprint_of(z)), "inputs differ from the reference run's"
    orc = Oracle(d)
    txs = sorted(int(k[2:-7]) for k in z.files if k.endswith("_traces"))
    assert txs == list(range(orc.NTx if case in ("txvar", "wide_142x36x25") else 1))
    for t in txs:
        got, n = orc.run(t)
        assert n == int(z[f"tx{t}_steps"])
        check(got, z[f"tx{t}_traces"], orc.nefcmp, 1e-10)


def test_oracle_halfspace_run_matches_the_reference_kernels():
    import gen_oracle_traces as g

    z = ref("halfspace_64x64x48")
    got, n, _, fp = g.load("halfspace_64x64x48")
    assert g.same_inputs(fp, g.fingerprint_of(z))
    assert n == int(z["tx0_steps"]) == 3026
    check(got, z["tx0_traces"], 2, 2e-8)


def first_400_steps(case):
    import gen_oracle_traces as g

    z = ref(case)
    got, n, max_steps, fp = g.load(case)
    assert g.same_inputs(fp, g.fingerprint_of(z))
    exp = z["tx0_traces"]
    reached = np.nonzero(np.abs(got).max(axis=(0, 1)))[0]
    k = int(reached[-1])  # samples before the last one the window reached are complete
    assert k >= 10
    return got[..., :k], exp[..., :k]


def test_oracle_first_400_steps_match_the_reference_kernels_1d_marine():
    got, exp = first_400_steps("marine1d_128x128x96")
    check(got, exp, 2, 1e-10)


def test_oracle_first_400_steps_match_the_reference_kernels_3d_marine():
    """On the 256 x 256 x 160 grid the reference's own runs differ from each other (see the
    module notes): three runs of 800 steps of marine3d_strip35_256x256x160 spread by up to
    1.7e-9 of the largest trace, while on 128 x 128 x 96 they agree to 4e-15.  The oracle is
    compared on that scale: 1e-8 of the largest trace of each field (measured 2.5e-9)."""
    got, exp = first_400_steps("marine3d_strip35_256x256x160")
    assert field_error(got, exp, 2) < 1e-8


def test_reference_run_with_280_point_strips_is_not_finite():
    """marine3d_256x256x160: the reference's traces are NaN, as the shared-memory reads of its
    strip kernels predict (see the module notes)."""
    z = ref("marine3d_256x256x160")
    assert not np.isfinite(z["tx0_traces"]).any()
    h = np.load(os.path.join(GOLDEN, "ref_host_marine3d_256x256x160.npz"))
    mp = dict(zip(["AnLx_old", "AnRx_old", "Any_old", "Anz", "ALx1", "ALx2", "ARx1", "ARx2", "Ay1", "Ay2", "Az1",
                   "Az2", "L", "M", "N", "Nx", "Ny", "Nz", "AnLx_New", "AnRx_New", "Any_New", "LNx2", "LMy2"],
                  (int(v) for v in h["mp_i"])))
    for pts, nodes in ((mp["AnLx_New"], mp["ALx1"] + mp["ALx2"] + 4), (mp["AnRx_New"], mp["ARx1"] + mp["ARx2"] + 4),
                       (mp["Any_New"], mp["Ay1"] + mp["Ay2"] + 4)):
        assert pts > 256 and pts % 256 < nodes
    s = np.load(os.path.join(GOLDEN, "ref_host_marine3d_strip35_256x256x160.npz"))["mp_i"]
    assert all(int(s[q]) <= 256 for q in (18, 19, 20))  # one block per strip
