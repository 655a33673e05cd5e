import os
import sys
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")
    config.addinivalue_line("markers", "slow: long-running parity case")


@pytest.fixture(scope="session")
def case_dir():
    """Factory: writes a named input case once per session and returns its directory."""
    from tcsem_fdtd_gb300 import inputs

    made = {}
    root = tempfile.mkdtemp(prefix="tcsem_cases_")

    def get(name, **overrides):
        key = (name, tuple(sorted((k, repr(v)) for k, v in overrides.items())))
        if key not in made:
            d = os.path.join(root, f"{name}_{len(made)}")
            inputs.write_case(inputs.case(name, **overrides), d)
            made[key] = d
        return made[key]

    return get


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
