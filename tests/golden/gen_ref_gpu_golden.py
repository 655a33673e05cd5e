"""Regenerate tests/golden/ref_gpu_<case>.npz: receiver traces computed by the reference's
own CUDA kernels.

Needs a GPU and the reference's kernels compiled into oracle/_ref/*.cubin by
oracle/build_ref.py (from the reference tree, in the container that has it); the
modules carry device code only, so they load on the GPU machine.  oracle/ref_gpu.py
drives them with the setup arrays of the reference's own host code
(tests/golden/ref_host_<case>.npz) and the seeded survey inputs.

Each file holds, per transmitter run, the traces, the step count and the device time of
the step loop, plus the fingerprint of the inputs (tests/golden/gen_oracle_traces.py;
tests check that their inputs are the same).  Only the first transmitter is defined in the reference itself (its
counters carry over between transmitters, main.cu:76-78,207); the other transmitters of
txvar and wide_142x36x25 are run the same way from a zero state, which pins the
reference's source injection for every orientation.

    python tests/golden/gen_ref_gpu_golden.py [--out DIR] [case ...]
"""
import argparse
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
from gen_oracle_traces import inputs_fingerprint  # noqa: E402
from oracle import ref_gpu  # noqa: E402
from tcsem_fdtd_gb300 import inputs  # noqa: E402

# case -> transmitters to run
CASES = {"tiny": [0], "small": [0], "txvar": [0, 1, 2, 3, 4, 5], "wide_142x36x25": [0, 1, 2],
         "halfspace_64x64x48": [0], "marine1d_128x128x96": [0], "marine3d_256x256x160": [0],
         "marine3d_strip35_256x256x160": [0]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE)
    ap.add_argument("cases", nargs="*")
    a = ap.parse_args()
    if not ref_gpu.cubins_present():
        raise SystemExit("oracle/_ref/*.cubin missing: run oracle/build_ref.py where the reference tree is")
    os.makedirs(a.out, exist_ok=True)
    summary = {}
    for case in a.cases or list(CASES):
        with tempfile.TemporaryDirectory() as d:
            inputs.write_case(inputs.case(case), d)
            digest, con_stats = inputs_fingerprint(d)
            rec = {"digest": digest, "con_stats": con_stats}
            for t in CASES[case]:
                tr, steps, ms = ref_gpu.run(d, os.path.join(HERE, f"ref_host_{case}.npz"), itx=t)
                rec[f"tx{t}_traces"] = tr
                rec[f"tx{t}_steps"] = steps
                rec[f"tx{t}_ms"] = ms
                summary[f"{case}/tx{t}"] = {"steps": steps, "ms": round(ms, 3), "peak": float(np.abs(tr).max()),
                                            "finite": bool(np.isfinite(tr).all())}
                print(case, t, summary[f"{case}/tx{t}"], flush=True)
        np.savez_compressed(os.path.join(a.out, f"ref_gpu_{case}.npz"), **rec)
        summary[case] = {"digest": digest}
    with open(os.path.join(a.out, "ref_gpu_summary.json"), "w") as f:
        json.dump(summary, f, indent=1)


if __name__ == "__main__":
    main()
