import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _oracle_built():
    """The CPU oracle (the project's C restatement) is test infrastructure:
    build it once per session if it is missing."""
    lib = os.path.join(ROOT, "oracle", "liborc.so")
    if not os.path.exists(lib):
        subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_oracle.sh")], check=True)
    yield


GOLDEN = os.path.join(ROOT, "tests", "golden")
