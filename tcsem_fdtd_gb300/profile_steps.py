"""Run a few time steps of a named synthetic workload, for profilers.

    python -m tcsem_fdtd_gb300.profile_steps [--workload marine3d_256x256x160] [--steps 16]
                                             [--precision 32] [--serial-boundary] [--fused N]
                                             [--batch N [--persistent]]

Writes the workload's input files to a temporary directory, opens it through
the C ABI and advances `--steps` steps (CUDA graphs of 8 steps), then exits.
With `--fused N` it instead launches the fused sweep alone N times
(tcsem_fused_step: every z-chunk of the default layout in one launch, the
launch bench.py times for the roofline).  With `--batch N` it advances a
batch of the first N generated surveys of the batched workload instead
(`--steps` steps, graph blocks of 8; with `--persistent` each block is one
launch of the persistent batch kernel).
It reports nothing about speed: time with bench.py, and use this under ncu to
get a launch list or a capture of one kernel on a short run.
"""
import argparse
import os
import sys
import tempfile

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main(argv=None):
    from tcsem_fdtd_gb300 import Simulation, inputs

    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="marine3d_256x256x160")
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--precision", type=int, default=32, choices=[32, 64])
    ap.add_argument("--serial-boundary", action="store_true",
                    help="boundary pipeline before one launch of the whole sweep (no overlap)")
    ap.add_argument("--fused", type=int, default=0, help="launch the fused sweep alone this many times")
    ap.add_argument("--batch", type=int, default=0, help="advance a batch of this many generated surveys")
    ap.add_argument("--persistent", action="store_true", help="the batch's persistent schedule (one launch per block)")
    a = ap.parse_args(argv)
    if a.batch:
        from tcsem_fdtd_gb300 import Batch

        root = tempfile.mkdtemp(prefix="tcsem_prof_batch_")
        dirs = []
        for q in range(a.batch):
            dq = os.path.join(root, f"s{q:03d}")
            inputs.write_case(inputs.batch_case(q), dq)
            dirs.append(dq)
        with Batch(precision=a.precision, graph_steps=8, persistent=a.persistent) as b:
            for dq in dirs:
                b.add(dq)
            b.advance(a.steps)
            b.poll()
        print(f"batch of {a.batch}: {a.steps} steps", flush=True)
        return 0
    d = tempfile.mkdtemp(prefix=f"tcsem_prof_{a.workload}_")
    inputs.write_case(inputs.case(a.workload), d)
    with Simulation(d, precision=a.precision, graph_steps=8, serial_boundary=a.serial_boundary) as sim:
        sim.begin(0)
        if a.fused:
            sc = sim.schedule()
            for q in range(a.fused):
                sim.fused_step(sc["lam"][q], sc["dt1"][q], 0.5 * (sc["dt1"][q] + sc["dt2"][q]), 0.0)
            sim.synchronize()
            print(f"{a.workload}: {a.fused} fused sweeps, {sim.info['zchunks']} z-chunks", flush=True)
            return 0
        sim.advance(a.steps)
        sim.synchronize()
        print(f"{a.workload}: {a.steps} steps, {sim.info['launches_per_step']} launches per step", flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
