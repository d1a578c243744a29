import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as G  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


@pytest.fixture(scope="session")
def pkg():
    return G.load_package()


@pytest.fixture(scope="session")
def synth(pkg):
    from gpu_intensities_gb300 import synth as S
    return S


@pytest.fixture(scope="session")
def oracle():
    O = G.load_oracle()
    O.lib()
    return O
