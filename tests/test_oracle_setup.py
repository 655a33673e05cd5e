"""The oracle's setup restatement against the reference's own host code.

The fixtures in tests/golden/ref_host_*.npz were produced by the reference's
ModelingSetup/Waveform/ModelGridMapping/LoadRxTxPos (tests/golden/gen_ref_host_golden.py).
Index maps and located cells must agree exactly; coordinates to within a few
ulps (libm pow/exp10 may differ by one ulp between hosts).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

CASES = ["tiny", "small", "txvar", "example", "halfspace_64x64x48", "marine1d_128x128x96", "marine3d_256x256x160",
         "wide_142x36x25", "marine3d_strip35_256x256x160"]


def load(name):
    return dict(np.load(os.path.join(GOLDEN, f"ref_host_{name}.npz")))


@pytest.mark.parametrize("name", CASES)
def test_grid_and_maps_match_reference_host(name, case_dir):
    from oracle.oracle import Oracle

    g = load(name)
    o = Oracle(case_dir(name))
    dims = g["dims"]
    assert [o.L, o.M, o.N, o.L1, o.M1, o.AnLx_New, o.AnRx_New, o.Any_New, o.NRx, o.NTx, o.Nt, o.NComp,
            o.nefcmp, o.nsrc, o.IsLog] == [int(v) for v in dims[:15]]
    for nm in ["dx", "dy", "dz", "X", "Y", "Z", "Xn", "Yn", "times", "dtw", "wave", "rx", "ry", "rz"]:
        np.testing.assert_allclose(o.darray(nm), g[nm], rtol=4e-15, atol=1e-300, err_msg=nm)
    for nm in ["xBzNew2old", "yBzNew2old", "xBzold2New", "yBzold2New", "xoldBx2NewBz", "yoldBy2NewBz",
               "rix", "riy", "riz"]:
        np.testing.assert_array_equal(o.iarray(nm), g[nm], err_msg=nm)
    p = g["params"]
    assert (o.sfa1, o.sfa2, o.sita_t, o.minsita) == tuple(p[:4])
    for t in range(o.NTx):
        iv, dv, rx = o.tx(t)
        giv = g[f"tx{t}_i"]
        set_ = giv >= 0
        np.testing.assert_array_equal(iv[set_], giv[set_], err_msg=f"tx{t}")
        np.testing.assert_allclose(dv, g[f"tx{t}_d"], rtol=1e-15, err_msg=f"tx{t}")
        np.testing.assert_array_equal(rx, g[f"tx{t}_rx"])


def test_waveform_matches_shipped_testwaveform():
    """Waveform() restated vs the reference's shipped testwaveform.dat (N=100, sigma_t=1e-3).

    The shipped file's bytes are reproduced by the reference's own code for the
    'example' case (its FDTD_setup.in has n1=200, sigma_t=1e-3); the fixture keeps
    those bytes and the oracle must match them.
    """
    from oracle.oracle import Oracle
    import tempfile
    from tcsem_fdtd_gb300 import inputs

    g = load("example")
    raw = g["testwaveform"].tobytes()
    n = int(np.frombuffer(raw[:4], np.int32)[0])
    a = np.frombuffer(raw[4:], np.float64)
    t, dt, w = a[:2 * n + 1], a[2 * n + 1:4 * n + 2], a[4 * n + 2:]
    d = tempfile.mkdtemp()
    inputs.write_case(inputs.case("example"), d)
    o = Oracle(d)
    np.testing.assert_array_equal(o.darray("tw"), t)
    np.testing.assert_array_equal(o.darray("dtw")[:2 * n + 1], dt)
    np.testing.assert_allclose(o.darray("wave"), w, rtol=1e-15)
