import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# The sledgehamr source tree (only where it is present, for the tests that
# pin the oracle to the reference's own code): $SLEDGEHAMR_REF_ROOT, else a
# directory named "reference" beside this repository.
REF_ROOT = os.environ.get("SLEDGEHAMR_REF_ROOT") or os.path.join(os.path.dirname(ROOT),
                                                                 "reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from tests.oracle_lib import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def ref():
    from tests.oracle_lib import Oracle, ref_available
    if not ref_available():
        pytest.skip("oracle/_ref not built (sledgehamr sources absent)")
    return Oracle(ref=True)


@pytest.fixture(scope="session")
def ctx():
    import sledgehamr_gb300 as sh
    c = sh.Context(0)
    yield c
    c.close()


def golden(name):
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"), allow_pickle=False)


def rel_l2(a, b):
    import numpy as np
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
