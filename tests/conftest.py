import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = sorted(d for d in os.listdir(GOLDEN) if os.path.isfile(os.path.join(GOLDEN, d, "golden.npz")))
# cases whose operators are rebuilt from rho by the e-e model (eeMode = Pee_update), and the others
# (the linearized e-e cases hold the e-e term inside their fixed linear operators)
EE_CASES = [c for c in GOLDEN_CASES if c.startswith("ee_") and "linear" not in c]
FIXED_P_CASES = [c for c in GOLDEN_CASES if c not in EE_CASES]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    O._setup_prototypes()
    return O


def pytest_collection_modifyitems(config, items):
    """The whole-run tests (DMD's time loop through the host library, which writes its output files)
    go after every other test; the order is otherwise unchanged."""
    items[:] = sorted(items, key=lambda it: "test_host_run.py::" in it.nodeid)
