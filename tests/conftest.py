import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")


@pytest.fixture(scope="session")
def golden():
    """Arrays written by tests/golden/make_golden.py from the reference itself."""
    with np.load(os.path.join(GOLDEN, "golden_small.npz")) as z:
        data = {k: z[k] for k in z.files}

    class G:
        def __call__(self, case):
            pre = case + "__"
            return {k[len(pre):]: v for k, v in data.items() if k.startswith(pre)}

    return G()


@pytest.fixture(scope="session")
def golden_hash():
    import json
    with open(os.path.join(GOLDEN, "golden_hash.json")) as f:
        return json.load(f)
