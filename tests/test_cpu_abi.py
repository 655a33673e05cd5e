"""CPU-side checks of the product library: it loads, exports every symbol the
header declares, validates its inputs, and fails loudly without a GPU."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT


def test_library_builds_and_exports_header_symbols():
    from tcsem_fdtd_gb300 import build

    build.build()
    import tcsem_fdtd_gb300 as t

    lib = t.library()
    names = t.declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_opts_and_info_struct_layout_matches_header():
    import tcsem_fdtd_gb300 as t
    from tcsem_fdtd_gb300.api import Info, Opts

    o = Opts()
    t.library().tcsem_default_opts(C.byref(o))
    assert o.precision == 32 and o.device == 0 and o.fix_dual_bipole == 0 and o.serial_boundary == 0
    assert C.sizeof(Opts) == 36 and o.persistent_batch == 0


def test_struct_offsets_match_the_c_compiler(tmp_path):
    """Every field of the records in include/tcsem.h sits where gcc puts it."""
    import shutil
    import subprocess

    from tcsem_fdtd_gb300.api import HEADER, Info, ModelRec, Opts, SurveyRec, TxRec

    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    lines = []
    records = ((Opts, "tcsem_opts"), (Info, "tcsem_info"), (ModelRec, "tcsem_model"), (TxRec, "tcsem_transmitter"),
               (SurveyRec, "tcsem_survey"))
    for st, cname in records:
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in st._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    src = tmp_path / "off.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "tcsem.h"\nint main(void) {\n' +
                   "\n".join(lines) + "\nreturn 0;\n}\n")
    exe = tmp_path / "off"
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        cname, f, v = ln.split()
        got[(cname, f)] = int(v)
    for st, cname in records:
        assert got[(cname, "sizeof")] == C.sizeof(st), cname
        for f, _ in st._fields_:
            assert got[(cname, f)] == getattr(st, f).offset, (cname, f)


def test_open_without_gpu_or_with_bad_inputs_fails_loudly(case_dir, tmp_path):
    import tcsem_fdtd_gb300 as t

    with pytest.raises(t.TcsemError):
        t.Simulation(str(tmp_path))  # no input files
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        with pytest.raises(t.TcsemError) as e:
            t.Simulation(case_dir("tiny"))
        assert e.value.status == 4  # TCSEM_ERR_CUDA, never a silent CPU path


def test_in_memory_open_checks_its_records_like_the_parser():
    """tcsem_open refuses what tcsem_open_dir refuses in a file, with the same codes, before it
    touches a GPU; a valid survey then stops at the device (TCSEM_ERR_CUDA without a GPU)."""
    import copy

    import tcsem_fdtd_gb300 as t
    from tcsem_fdtd_gb300 import inputs

    model, survey = inputs.memory_case(inputs.case("txvar"))
    bad = copy.deepcopy(survey)
    bad["tx"][2]["ort"] = 7
    with pytest.raises(t.TcsemError) as e:
        t.Simulation(model=model, survey=bad)
    assert e.value.status == 2 and "orientation" in str(e.value)
    bad = copy.deepcopy(survey)
    bad["tx"][0]["rx"] = [1, 6]  # five receivers
    with pytest.raises(t.TcsemError) as e:
        t.Simulation(model=model, survey=bad)
    assert e.value.status == 2 and "receiver id" in str(e.value)
    m2 = dict(model, ALx1=0, ALx2=0)
    with pytest.raises(t.TcsemError) as e:
        t.Simulation(model=m2, survey=survey)
    assert e.value.status == 3
    for bad_grid in (dict(ALx2=-1, Nx=model["Nx"] + 1), dict(Ny=0, Ay1=model["Ay1"] + 1), dict(dzmin=0.0)):
        with pytest.raises(t.TcsemError) as e:
            t.Simulation(model=dict(model, **bad_grid), survey=survey)
        assert e.value.status == 3 and "grid" in str(e.value), bad_grid
    with pytest.raises(t.TcsemError) as e:
        t.Simulation(model=model, survey=dict(survey, Nt=1))
    assert e.value.status == 3 and "sampling times" in str(e.value)
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        with pytest.raises(t.TcsemError) as e:
            t.Simulation(model=model, survey=survey)
        assert e.value.status == 4 and "CUDA device" in str(e.value)


def test_parse_errors_are_reported(tmp_path):
    import tcsem_fdtd_gb300 as t
    from tcsem_fdtd_gb300 import inputs

    d = str(tmp_path / "bad")
    inputs.write_case(inputs.case("tiny"), d)
    with open(os.path.join(d, "Transmitter.in"), "w") as f:
        f.write("1\n1 7 100.0 0.0 0.0 20.0 1 1\n")  # illegal orientation 7
    with pytest.raises(t.TcsemError) as e:
        t.Simulation(d)
    assert e.value.status == 2
    os.remove(os.path.join(d, "Cond.bin"))
    with pytest.raises(t.TcsemError) as e:
        t.Simulation(d)
    assert e.value.status == 1


def test_cli_usage_error_exit_code():
    from tcsem_fdtd_gb300 import build

    build.build()
    r = subprocess.run([build.CLI, "--bogus"], capture_output=True, text=True)
    assert r.returncode == 2


def test_integration_snippets_compile_against_the_header(tmp_path):
    """The C code of the integration guide at the repository root compiles against
    include/tcsem.h and links against the library's exported symbols (gcc; the snippets placed
    in a main())."""
    import re
    import shutil
    import subprocess

    from tcsem_fdtd_gb300.api import HEADER

    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    text = open(os.path.join(os.path.dirname(HEADER), "..", "INTEGRATION.md")).read()
    blocks = re.findall(r"```c\n(.*?)```", text, flags=re.S)
    assert len(blocks) >= 2
    body = "\n".join(b for b in blocks if "#include" not in b)
    first = next(b for b in blocks if "#include" in b)
    src = tmp_path / "snippet.c"
    src.write_text("#include <stdio.h>\n#include <stdlib.h>\n" + first.split("\n", 1)[0] + "\n"
                   "int main(void) {\n" + first.split("\n", 1)[1] + "\n{\n" + body + "\n}\nreturn 0;\n}\n")
    lib_dir = os.path.dirname(__import__("tcsem_fdtd_gb300").api.LIB_PATH)
    cmd = ["gcc", "-std=c99", "-Wall", "-Werror", "-Wno-unused-variable", "-I", os.path.dirname(HEADER), str(src)]
    if os.path.exists(os.path.join(lib_dir, "libtcsem.so")):  # link against the exported symbols
        cmd += ["-o", str(tmp_path / "snippet"), "-L", lib_dir, "-ltcsem"]
    else:  # compile only
        cmd += ["-c", "-o", str(tmp_path / "snippet.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_integration_guide_covers_every_entry_point():
    """Every function include/tcsem.h declares is described in the integration guide."""
    from tcsem_fdtd_gb300.api import HEADER, declared_functions

    doc = open(os.path.join(os.path.dirname(HEADER), "..", "INTEGRATION.md")).read()
    missing = [f for f in declared_functions() if f not in doc]
    assert not missing, missing
