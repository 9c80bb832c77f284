import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_port():
    """The plain-C oracle restatement, built on first use."""
    from oracle import oracle as O
    O.build("port")
    return O.OracleLib("port")


@pytest.fixture(scope="session")
def oracle_ref():
    """The reference compiled in place; skipped where its sources are absent."""
    from oracle import oracle as O
    if not O.ref_available():
        if not os.path.isdir(O.REF_SRC):
            pytest.skip("reference sources not present on this machine")
        O.build("ref")
    return O.OracleLib("ref")
