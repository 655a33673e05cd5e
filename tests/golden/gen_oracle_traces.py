"""Regenerate tests/golden/oracle_traces_<case>.npz: receiver traces of the FP64 oracle.

The oracle (oracle/tcsem_oracle.c) takes minutes on the larger survey grids, so its traces
of these runs are stored once and the GPU tests compare the CUDA path against them:

* halfspace_64x64x48   -- the whole run (3026 steps), transmitter 1;
* marine1d_128x128x96  -- the first 400 steps (source window and the first samples);
* marine3d_256x256x160 -- the first 400 steps;
* marine3d_strip35_256x256x160 -- the first 400 steps.

Each file holds the traces (trimmed after the last sample the run reached), the step count,
and a fingerprint of the inputs the seeded generator wrote, so a test can tell whether its
inputs are the ones the traces were computed from: the SHA-256 of the three text files and
three sums over the conductivity, compared to 1e-10 (numpy's exp and log may round the last
bit differently on another CPU architecture; a different random stream changes the sums at
the percent level).

    python tests/golden/gen_oracle_traces.py [case ...]
"""
import hashlib
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle.oracle import Oracle  # noqa: E402
from tcsem_fdtd_gb300 import inputs  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
RUNS = {"halfspace_64x64x48": -1, "marine1d_128x128x96": 400, "marine3d_256x256x160": 400,
        "marine3d_strip35_256x256x160": 400}
INPUT_FILES = ("FDTD_setup.in", "Cond.bin", "Receiver.in", "Transmitter.in")


def inputs_fingerprint(directory):
    """(SHA-256 of FDTD_setup.in, Receiver.in and Transmitter.in; [sum, sum of squares,
    index-weighted sum] of the conductivity in Cond.bin)."""
    h = hashlib.sha256()
    for f in INPUT_FILES:
        if f == "Cond.bin":
            continue
        with open(os.path.join(directory, f), "rb") as fh:
            h.update(fh.read())
    con = np.fromfile(os.path.join(directory, "Cond.bin"), dtype="<f8")
    w = np.linspace(1.0, 2.0, con.size)
    return h.hexdigest(), np.array([con.sum(), (con * con).sum(), (con * w).sum()])


def same_inputs(fa, fb):
    return fa[0] == fb[0] and np.allclose(fa[1], fb[1], rtol=1e-10, atol=0.0)


def fingerprint_of(z):
    """The inputs fingerprint stored in a fixture file."""
    return str(z["digest"]), np.asarray(z["con_stats"])


def path(case):
    return os.path.join(HERE, f"oracle_traces_{case}.npz")


def load(case):
    """(traces padded back to the full sample count, steps, max_steps, inputs fingerprint)."""
    z = np.load(path(case))
    tr = z["traces"]
    full = np.zeros(tuple(z["shape"]))
    full[..., : tr.shape[2]] = tr
    return full, int(z["nsteps"]), int(z["max_steps"]), fingerprint_of(z)


def generate(case):
    max_steps = RUNS[case]
    with tempfile.TemporaryDirectory() as d:
        inputs.write_case(inputs.case(case), d)
        digest, con_stats = inputs_fingerprint(d)
        orc = Oracle(d)
        tr, n = orc.run(0, max_steps=max_steps)
        orc.close()
    nz = np.nonzero(np.abs(tr).max(axis=(0, 1)))[0]
    keep = int(nz[-1]) + 1 if len(nz) else 0
    np.savez_compressed(path(case), traces=tr[..., :keep], shape=np.array(tr.shape), nsteps=n,
                        max_steps=max_steps, digest=digest, con_stats=con_stats)
    print(f"{case}: {n} steps, {keep} of {tr.shape[2]} samples reached, inputs {digest[:16]}")


if __name__ == "__main__":
    for c in sys.argv[1:] or list(RUNS):
        generate(c)
