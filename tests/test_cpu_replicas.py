"""The multi-process path of bench.py on CPU: ranks started by torch.distributed.run
with the gloo backend (one independent replica per rank, no data-path
collective; the ranks only meet for barriers and the max/sum of their timings).
"""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _ranks(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist()
    d.barrier()
    q.put((rank, d.reduce(10.0 + rank, "max"), d.reduce(1.0 + rank, "sum")))
    d.close()


def test_rank_reductions_with_gloo():
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = free_port()
    ps = [mp.Process(target=_ranks, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 11.0, 3.0), (1, 11.0, 3.0)]


def test_reference_arm_under_torchrun_two_ranks():
    """Rank 0 alone runs the CPU reference arm and prints one JSON line; rank 1 exits 0 without work."""
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--workload", "tiny", "--gpus", "2", "--steps", "4", "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(ln) for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["config"]["workload"] == "tiny" and len(line["config"]["plane"]) == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_bench_helpers_on_the_host():
    """The figures bench.py reads from committed files (the sweep's ncu traffic, the measured HBM
    peak) and the reference CPU-remap record, which is either a timing or says why it is absent."""
    sys.path.insert(0, ROOT)
    import bench
    from tcsem_fdtd_gb300 import inputs

    t = bench.profiled_traffic("marine3d_256x256x160")
    assert t is None or 5e8 < t < 7e8  # 575 MB per launch; about 52 B x 10.5 M cells
    peak, kind = bench.measured_peak()
    assert peak > 1000 and kind in ("measured", "fallback")
    d = bench.make_inputs("tiny", 0)
    rec = bench.reference_cpu_remap(d, reps=2)
    if rec is not None:
        L1, M1 = rec["plane"]
        assert rec["ms_per_call"] > 0 and L1 > 0 and M1 > 0 and rec["kind"] == "reference"
