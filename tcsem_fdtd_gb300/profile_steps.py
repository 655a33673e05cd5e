"""Run a few time steps of a named synthetic workload, for profilers.

    python -m tcsem_fdtd_gb300.profile_steps [--workload cfg3] [--steps 16]
                                             [--precision 32] [--serial-boundary]

Writes the workload's input files to a temporary directory, opens it through
the C ABI and advances `--steps` steps (CUDA graphs of 8 steps), then exits.
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
    ap.add_argument("--workload", default="cfg3")
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--precision", type=int, default=32, choices=[32, 64])
    ap.add_argument("--serial-boundary", action="store_true",
                    help="boundary pipeline before one launch of the whole sweep (no overlap)")
    a = ap.parse_args(argv)
    d = tempfile.mkdtemp(prefix=f"tcsem_prof_{a.workload}_")
    inputs.write_case(inputs.case(a.workload), d)
    with Simulation(d, precision=a.precision, graph_steps=8, serial_boundary=a.serial_boundary) as sim:
        sim.begin(0)
        sim.advance(a.steps)
        sim.synchronize()
        print(f"{a.workload}: {a.steps} steps, {sim.info['launches_per_step']} launches per step", flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
