import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "simple-vector-db_gb300")
for p in (os.path.join(ROOT, "oracle"), PKG, os.path.join(ROOT, "tests", "golden"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


_PARITY_LINES = []


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def parity_report():
    """Lines describing what a parity test checked (sample sizes, the
    screen's certification statistics), printed at the end of the run."""
    return _PARITY_LINES


def pytest_terminal_summary(terminalreporter, exitstatus, config):
    if _PARITY_LINES:
        terminalreporter.write_sep("-", "parity at the measured sizes")
        for line in _PARITY_LINES:
            terminalreporter.write_line(line)


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build(ref=False)
    return O.Oracle()


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "golden_reference.npz")))


@pytest.fixture(scope="session")
def svdb():
    """The library binding; built here if missing (CPU build works: nvcc
    cross-compiles sm_103a)."""
    lib = os.path.join(PKG, "_build", "libsvdb_gb300.so")
    if not os.path.isfile(lib):
        sys.path.insert(0, PKG)
        import build as B
        B.build()
    import svdb_gb300
    return svdb_gb300


@pytest.fixture(scope="session")
def refstore():
    """The reference's own compiled store, where its sources exist."""
    import oracle as O
    if not os.path.isfile(O.REF_SO):
        if os.path.isdir(os.path.join(O.REF_SRC, "src")):
            O.build(ref=True)
        else:
            pytest.skip("reference sources not present")
    return O.RefLib()
