"""Test configuration.

Markers:
  gpu -- needs a CUDA device (run with `-m gpu` on a GB300); everything else
         runs on the CPU.
The checkers (oracle/liboracle.so) and the product library
(qcs_gb300/libqcs_gb300.so) are built on first use.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from oracle import oracle as O
    from qcs_gb300 import build as B
    O.build()
    B.build()
    yield


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    d = os.path.join(ROOT, "tests", "golden")

    def load(name):
        return dict(np.load(os.path.join(d, name + ".npz")))
    return load
