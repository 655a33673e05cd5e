"""tcsem_upcontinuation_noalloc (static scratch, no allocation at call time)
against tcsem_upcontinuation (the handle's own work arrays), through the C ABI.

The two run the same kernels on the same inputs, so the results agree to the
last bit in practice; the check allows 1e-12 (FP64) / 1e-6 (FP32) relative to
the largest value.  Each entry point is called twice in a row on the same
input, which also shows that a second call over scratch left by the first
(or by earlier tests in the same process) changes nothing.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {64: 1e-12, 32: 1e-6}


@pytest.fixture(scope="module")
def lib():
    from tcsem_fdtd_gb300 import build, library

    build.build()
    return library()


def boundary_twice(lib, sim, fn, bz):
    out = []
    for _ in range(2):
        sim.set("Bz", bz)
        sim.set("BxAir", np.zeros(sim.field_shape("BxAir")))
        sim.set("ByAir", np.zeros(sim.field_shape("ByAir")))
        st = getattr(lib, fn)(sim._h)
        assert st == 0, lib.tcsem_last_error(sim._h).decode()
        assert lib.tcsem_synchronize(sim._h) == 0
        out.append((sim.get("BxAir"), sim.get("ByAir")))
    return out


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("name", ["small", "halfspace_64x64x48", "marine3d_256x256x160"])
def test_noalloc_boundary_matches_allocating_entry(lib, case_dir, name, precision):
    from tcsem_fdtd_gb300 import Simulation

    with Simulation(case_dir(name), precision=precision) as sim:
        bz = np.random.default_rng(21).standard_normal(sim.field_shape("Bz"))
        ref = boundary_twice(lib, sim, "tcsem_upcontinuation", bz)
        got = boundary_twice(lib, sim, "tcsem_upcontinuation_noalloc", bz)
    scale = max(np.abs(ref[0][0]).max(), np.abs(ref[0][1]).max())
    assert scale > 0
    for call in range(2):
        for comp in range(2):
            err = np.abs(got[call][comp] - ref[0][comp]).max() / scale
            assert err <= TOL[precision], (call, comp, err)


def test_noalloc_refuses_a_plane_beyond_the_static_scratch(lib, case_dir):
    """A 992 x 992 plane over 512 rows needs about 25 MB of FP64 scratch (> 16 MiB)."""
    from tcsem_fdtd_gb300 import Simulation, TcsemError

    d = case_dir("marine3d_256x256x160", xsplit=(0, 40, 432, 40, 0), ysplit=(0, 40, 432), zsplit=(0, 4, 44),
                 model=dict(kind="uniform", sigma=1.0))
    with Simulation(d, precision=64) as sim:
        assert (sim.info["L1"], sim.info["M1"]) == (992, 992)
        with pytest.raises(TcsemError) as e:
            sim.upcontinuation_noalloc()
        assert e.value.status == 3 and "static scratch holds 16777216" in str(e.value)
        sim.upcontinuation()  # the allocating entry point still serves it
        sim.synchronize()
