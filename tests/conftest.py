import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
REFERENCE = os.environ.get("CHIMES_REF_DIR", "/root/reference")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def cg():
    pkg = importlib.import_module("chimes_lsq-myllfork_gb300")
    if not os.path.exists(pkg.LIB_PATH):
        pkg.build()
    return pkg


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    if not os.path.exists(o.LIB):
        o.build()
    return o


def fixture_dir(name):
    return os.path.join(GOLDEN, name)


FIXTURES = ["water2b", "water3b", "ch4b", "small4b", "watercoul", "multifile", "skipframes", "hierarc", "tersoff",
            "invr", "notrans", "specific", "exclude", "chebyfix_zero", "chebyfix_const", "chebyfix_smooth"]


def frame_part(model, ref):
    """(A, b) of a reference fixture without the charge-constraint rows that a
    FITCOUL fit appends after its last frame, and those rows (A, b)."""
    _, nc = model.charge_columns()
    A, b = ref["A"], ref["b"]
    n = A.shape[0] - nc
    return A[:n], b[:n], A[n:], b[n:]
