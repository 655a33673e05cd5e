"""Checkpoint of a run in progress (tcsem_save_state / tcsem_load_state).

A run stopped after an arbitrary number of steps, saved, loaded into a new
handle of the same survey and continued gives the traces of the uninterrupted
run bit for bit (both precisions, the overlapped and the serial step order,
one and several z-chunks); a state is refused by a handle of another survey or
under another continuation plane or dual-bipole option, and a file that is not a saved
state is reported.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built():
    from tcsem_fdtd_gb300 import build

    build.build()
    return True


@pytest.mark.parametrize("precision,zchunks,serial", [(64, 0, False), (32, 0, False), (64, 4, True), (32, 1, False)])
def test_resumed_run_equals_the_uninterrupted_run(built, case_dir, tmp_path, precision, zchunks, serial):
    from tcsem_fdtd_gb300 import Simulation

    d = case_dir("small")
    kw = dict(precision=precision, zchunks=zchunks, serial_boundary=serial)
    path = tmp_path / "state.bin"
    with Simulation(d, **kw) as a:
        n, nr = a.info["nsteps"], a.info["NRx"]
        full = a.run(0)
        a.begin(0)
        a.advance(n // 3 + 1)  # stops inside a graph block
        a.save_state(path)
        a.advance(n)
        assert np.array_equal(a.traces(nr), full)
    with Simulation(d, **kw) as b:
        b.load_state(path)
        assert b.advance(n)
        assert np.array_equal(b.traces(nr), full)


def test_a_state_is_refused_by_another_survey(built, case_dir, tmp_path):
    from tcsem_fdtd_gb300 import Simulation, TcsemError

    path = tmp_path / "state.bin"
    with Simulation(case_dir("tiny"), precision=32) as a:
        a.begin(0)
        a.advance(10)
        a.save_state(path)
    with Simulation(case_dir("small"), precision=32) as b:
        with pytest.raises(TcsemError) as e:
            b.load_state(path)
        assert e.value.status == 3  # TCSEM_ERR_INVALID
        junk = tmp_path / "junk.bin"
        junk.write_bytes(b"not a state" * 20)
        with pytest.raises(TcsemError) as e:
            b.load_state(junk)
        assert e.value.status == 2  # TCSEM_ERR_PARSE
        b.run(0)  # the handle stays usable


@pytest.mark.parametrize("option", [dict(padded_plane=2), dict(fix_dual_bipole=True)])
def test_a_state_is_refused_under_other_physics_options(built, case_dir, tmp_path, option):
    """Same survey, precision and z-chunk layout, but a continuation plane or a source that
    differs: the saved state would continue under other physics, so it is refused."""
    from tcsem_fdtd_gb300 import Simulation, TcsemError

    d = case_dir("txvar")
    path = tmp_path / "state.bin"
    with Simulation(d, precision=32, zchunks=2) as a:
        a.begin(0)
        a.advance(10)
        a.save_state(path)
    with Simulation(d, precision=32, zchunks=2, **option) as b:
        with pytest.raises(TcsemError) as e:
            b.load_state(path)
        assert e.value.status == 3  # TCSEM_ERR_INVALID
        assert b.run(0).shape[0] >= 1  # the handle stays usable
