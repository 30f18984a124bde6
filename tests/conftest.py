"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Builds the library (nvcc cross-compiles without a GPU) and the oracle."""
    from smatranem_gb300 import build as B
    import oracle
    B.build()
    oracle.build()
    return True


@pytest.fixture(scope="session")
def port(built):
    import oracle
    return oracle.Oracle("port")


@pytest.fixture(scope="session")
def reference(built):
    import oracle
    if not oracle.reference_available():
        pytest.skip("reference sources not present: oracle/_ref not built")
    return oracle.Oracle("reference")


def golden_cases():
    """The time-loop fixtures (the mode-solver and S-matrix fixtures, modes_*.npz
    and scalc_*.npz, have their own tests)."""
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith(("modes_", "scalc_")))


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}
