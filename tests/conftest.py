import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN_DIR, "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def acor_series():
    z = np.load(os.path.join(GOLDEN_DIR, "acor_series.npz"))
    return {k: z[k] for k in z.files}


def acor_matrix(series, n, how):
    """The 2 x n matrices of nvidia_gtx_test.clj:325-346: row 0 the series, row 1
    twice it ("times 2") or one more ("plus 1")."""
    d = series["n%d" % n].astype(np.float32)
    r1 = d * np.float32(2) if how == "times 2" else d + np.float32(1)
    return np.stack([d, r1.astype(np.float32)])


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O
