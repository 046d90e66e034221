import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


_CASES = {}


def make_case(tmp_root, name, **over):
    """Case directory for preset `name` with overrides, cached per session."""
    from rocketcombustor_gb300 import cases

    key = (name, tuple(sorted(over.items())))
    if key not in _CASES:
        tag = name + "".join(f"_{k}{v}" for k, v in sorted(over.items()))
        d = os.path.join(str(tmp_root), tag)
        cases.make_case(d, name, **over)
        _CASES[key] = d
    return _CASES[key]


@pytest.fixture(scope="session")
def case_root(tmp_path_factory):
    return tmp_path_factory.mktemp("cases")


@pytest.fixture(scope="session")
def case_t1(case_root):
    return make_case(case_root, "t1")


@pytest.fixture(scope="session")
def case_t2(case_root):
    return make_case(case_root, "t2")
