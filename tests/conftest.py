import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("", "oracle", "scikit-fem-native_gb300"):
    path = os.path.join(ROOT, sub) if sub else ROOT
    if path not in sys.path:
        sys.path.insert(0, path)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture
def golden():
    return load_golden


@pytest.fixture(scope="session")
def surrogate():
    """The learned neo-Hookean closure trained by the default recipe (2M samples,
    3000 Adam steps, L-BFGS on 524,288 samples); trained once per test session."""
    sk = pytest.importorskip("skfemntv_gb300")
    return sk.EnergySurrogate.train(mu=1.0, lmbda=10.0, sigma=0.1, seed=1)
