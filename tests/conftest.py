import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300)")


@pytest.fixture(scope="session")
def case_dirs(tmp_path_factory):
    """The small generated cases the oracle finishes in seconds."""
    from madwave3_gb300.host import generator
    base = tmp_path_factory.mktemp("cases")
    out = {}
    for name in ("tiny_j0", "tiny_j3", "tiny_e2"):
        d = str(base / name)
        generator.write_case(d, **generator.CASES[name])
        out[name] = d
    return out


@pytest.fixture(scope="session")
def runs(case_dirs):
    from madwave3_gb300.host import setup
    return {k: setup.load(os.path.join(d, "input.dat")) for k, d in case_dirs.items()}
