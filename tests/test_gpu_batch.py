"""Batched form: several surveys of different sizes advanced together.

Each slot's traces must equal the same survey run alone through
tcsem_run with the same z-chunk layout (one chunk, the batch default; the
batched launches run the same per-CTA code on the same data): the check allows
1e-12 (FP64) / 1e-6 (FP32) relative to each trace's peak.
Slots join while others run and leave when done; admission respects the
device-memory budget.
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


def alone(d, precision, itx=0):
    from tcsem_fdtd_gb300 import Simulation

    with Simulation(d, precision=precision, zchunks=1) as sim:
        return sim.run(itx)


def run_to_end(b, block=64, limit=100000):
    done = set()
    for _ in range(limit):
        if b.stats()["running"] == 0:
            break
        b.advance(block)
        done.update(b.poll())
    return done


@pytest.mark.parametrize("precision", [64, 32])
def test_batch_equals_each_survey_alone(built, case_dir, precision):
    from tcsem_fdtd_gb300 import Batch

    cases = [("tiny", 0), ("small", 0), ("txvar", 3), ("halfspace_64x64x48", 0)]
    dirs = [(case_dir(n), itx) for n, itx in cases]
    with Batch(precision=precision) as b:
        slots = [b.add(d, itx) for d, itx in dirs]
        st = b.stats()
        assert st["slots"] == 4 and st["running"] == 4 and st["device_bytes"] > 0
        done = run_to_end(b)
        assert done == set(slots)
        for (d, itx), s in zip(dirs, slots):
            info = b.info(s)
            assert info["steps_done"] == info["nsteps"]
            exp = alone(d, precision, itx)
            got = b.traces(s, nr=exp.shape[0])
            assert np.all(np.isfinite(got))
            assert rel_err(got, exp) <= TOL[precision], (d, itx)


def test_slots_join_and_leave_between_blocks(built, case_dir):
    """A survey that joins while another runs, and one that leaves early, give the same traces."""
    from tcsem_fdtd_gb300 import Batch

    d1, d2, d3 = case_dir("small"), case_dir("tiny"), case_dir("txvar")
    with Batch(precision=32, graph_steps=32) as b:
        s1 = b.add(d1)
        s3 = b.add(d3, 1)
        b.advance(96)  # three blocks of s1 and s3 alone
        s2 = b.add(d2)  # joins at the next block
        b.advance(64)
        b.remove(s3)  # leaves before its run ends
        done = run_to_end(b, block=32)
        assert {s1, s2} <= done
        for d, s in ((d1, s1), (d2, s2)):
            exp = alone(d, 32)
            assert rel_err(b.traces(s, nr=exp.shape[0]), exp) <= TOL[32]
        b.remove(s1)
        b.remove(s2)
        assert b.stats()["slots"] == 0


def test_batch_with_the_padded_plane(built, case_dir):
    """Slots carry the batch's options: a padded continuation plane (mode 2) gives the same
    traces in the batch as alone."""
    from tcsem_fdtd_gb300 import Batch, Simulation

    dirs = [case_dir("small"), case_dir("halfspace_64x64x48")]
    with Batch(precision=32, padded_plane=2) as b:
        slots = [b.add(d) for d in dirs]
        run_to_end(b)
        for d, s in zip(dirs, slots):
            with Simulation(d, precision=32, zchunks=1, padded_plane=2) as sim:
                exp = sim.run(0)
            assert rel_err(b.traces(s, nr=exp.shape[0]), exp) <= TOL[32], d


def test_batch_layout_autotuner(built, case_dir):
    """zchunks = -1: the batch times a few z-chunk layouts on its first block, restarts the
    slots and keeps the fastest; each slot's traces equal the survey run alone with the
    layout the slot reports."""
    from tcsem_fdtd_gb300 import Batch

    dirs = [case_dir("small"), case_dir("tiny"), case_dir("halfspace_64x64x48")]
    with Batch(precision=32, zchunks=-1) as b:
        slots = [b.add(d) for d in dirs]
        run_to_end(b)
        for d, s in zip(dirs, slots):
            info = b.info(s)
            assert 1 <= info["zchunks"] <= 3
            top = info["top_planes"] if info["top_planes"] > 0 else -1
            from tcsem_fdtd_gb300 import Simulation

            with Simulation(d, precision=32, zchunks=info["zchunks"], top_planes=top) as sim:
                exp = sim.run(0)
            assert rel_err(b.traces(s, nr=exp.shape[0]), exp) <= TOL[32], (d, info["zchunks"], top)


def test_admission_by_device_budget(built, case_dir):
    from tcsem_fdtd_gb300 import Batch, TcsemError

    with Batch(precision=32, budget=1 << 20) as b:  # 1 MiB: not even the tiny survey fits
        with pytest.raises(TcsemError) as e:
            b.add(case_dir("tiny"))
        assert e.value.status == 5 and "budget" in str(e.value)
        assert b.stats()["slots"] == 0


def test_cli_batch_mode_writes_the_same_files(built, case_dir, tmp_path):
    """tcsem_fdtd --batch (all transmitters as one batch, with either schedule) writes the same
    Tx<k>.bout as the serial CLI."""
    import shutil
    import subprocess

    from tcsem_fdtd_gb300 import build

    out = {}
    flags = {"serial": [], "batch": ["--batch"], "persistent": ["--batch", "--persistent"]}
    for mode in flags:
        d = tmp_path / mode
        shutil.copytree(case_dir("txvar"), d)
        args = [build.CLI, str(d)] + flags[mode]
        r = subprocess.run(args, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out[mode] = {}
        for k in range(1, 7):
            raw = open(d / f"Tx{k}.bout", "rb").read()
            hdr = tuple(int(v) for v in np.frombuffer(raw[:12], np.int32))
            out[mode][k] = (hdr, np.frombuffer(raw[12:], np.float64).reshape(hdr))
    for k in range(1, 7):
        (h1, a), (h2, b), (h3, c) = out["serial"][k], out["batch"][k], out["persistent"][k]
        assert h1 == h2 == h3
        assert rel_err(b, a) <= 1e-4  # FP32; one z-chunk per batch slot vs the single-survey layout
        assert rel_err(c, b) <= 1e-6  # the same slots under the two schedules
