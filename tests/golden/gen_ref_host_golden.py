"""Regenerate tests/golden/ref_host_<case>.npz from the reference's own host code.

Runs oracle/_ref/ref_host (built by oracle/build_ref.py from the reference's
ModelingSetup.cpp, SourceWave.cpp, ModelGridMapping.cpp, LoadRxTxPos.cpp,
logspace.cpp and AuxiliaryMemory.cpp) on the seeded inputs of each case and
stores every array it reports.  Needs the reference source tree; hosts without it
use the committed .npz files.

    python tests/golden/gen_ref_host_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import build_ref  # noqa: E402
from tcsem_fdtd_gb300 import inputs  # noqa: E402

CASES = ["tiny", "small", "txvar", "example", "halfspace_64x64x48", "marine1d_128x128x96", "marine3d_256x256x160",
         "wide_142x36x25", "marine3d_strip35_256x256x160"]


def read_records(path):
    out = {}
    b = open(path, "rb").read()
    p = 0
    while p < len(b):
        n = int(np.frombuffer(b, np.int32, 1, p)[0]); p += 4
        name = b[p:p + n].decode(); p += n
        kind = chr(b[p]); p += 1
        cnt = int(np.frombuffer(b, np.int32, 1, p)[0]); p += 4
        dt = np.float64 if kind == "d" else np.int32
        out[name] = np.frombuffer(b, dt, cnt, p).copy(); p += cnt * np.dtype(dt).itemsize
    return out


def main():
    exe = build_ref.build_ref_host(verbose=True)
    if exe is None:
        print("reference tree absent; keeping the committed fixtures")
        return 0
    here = os.path.dirname(os.path.abspath(__file__))
    for name in CASES:
        with tempfile.TemporaryDirectory() as d:
            inputs.write_case(inputs.case(name), d)
            rec = os.path.join(d, "records.bin")
            r = subprocess.run([exe, d, rec], capture_output=True, text=True)
            if r.returncode != 0:
                raise SystemExit(f"{name}: ref_host failed: {r.stdout}\n{r.stderr}")
            arrays = read_records(rec)
            wf = os.path.join(d, "testwaveform.dat")
            if os.path.exists(wf):
                arrays["testwaveform"] = np.frombuffer(open(wf, "rb").read(), np.uint8).copy()
                shipped = os.path.join(build_ref.REF, "testwaveform.dat")
                if name == "example" and os.path.exists(shipped):
                    # the example case has the shipped FDTD_setup.in's n1 and sigma_t
                    assert open(shipped, "rb").read() == open(wf, "rb").read(), "waveform differs from shipped file"
        np.savez_compressed(os.path.join(here, f"ref_host_{name}.npz"), **arrays)
        print(name, {k: v.shape for k, v in arrays.items() if k in ("dims", "Xn", "Yn")})
    return 0


if __name__ == "__main__":
    sys.exit(main())
