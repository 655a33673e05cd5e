"""The in-memory open (tcsem_open) against the file open (tcsem_open_dir) of the same survey:
the same handle state, so the same traces bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built():
    from tcsem_fdtd_gb300 import build

    build.build()
    return True


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("name", ["tiny", "txvar", "wide_142x36x25"])
def test_in_memory_open_equals_file_open(built, case_dir, name, precision):
    from tcsem_fdtd_gb300 import Simulation, inputs

    model, survey = inputs.memory_case(inputs.case(name))
    with Simulation(case_dir(name), precision=precision) as a, \
            Simulation(model=model, survey=survey, precision=precision) as b:
        for k in ("L", "M", "N", "L1", "M1", "NRx", "NTx", "Nt", "NComp", "nsteps", "zchunks", "top_planes",
                  "uploaded_bytes", "device_bytes"):
            assert a.info[k] == b.info[k], k
        np.testing.assert_array_equal(a.get("Con"), b.get("Con"))
        for k, v in a.schedule().items():
            np.testing.assert_array_equal(v, b.schedule()[k], err_msg=k)
        for itx in range(a.info["NTx"]):
            np.testing.assert_array_equal(a.run(itx), b.run(itx), err_msg=f"tx{itx}")
