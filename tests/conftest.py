import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = sorted(d for d in os.listdir(GOLDEN) if os.path.isfile(os.path.join(GOLDEN, d, "golden.npz")))
# cases whose operators are rebuilt from rho by the e-e model (eeMode = Pee_update), and the others
EE_CASES = [c for c in GOLDEN_CASES if c.startswith("ee_")]
FIXED_P_CASES = [c for c in GOLDEN_CASES if not c.startswith("ee_")]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    O._setup_prototypes()
    return O
