import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


def pytest_collection_modifyitems(config, items):
    """Unit-level parity first, then the end-to-end methane chains (files named *golden*),
    then the files named to run last (test_zz_*): under -x a failure in a long end-to-end
    chain does not keep the unit parity results from being reported.  Order within each
    group is the collection order."""

    def group(item):
        name = os.path.basename(str(item.fspath))
        if name.startswith("test_zz_"):
            return 2
        return 1 if "golden" in name else 0

    items[:] = sorted(items, key=group)


def is_approx(a, b, prec):
    """Eigen's isApprox: ||a - b|| <= prec * min(||a||, ||b||)."""
    import numpy as np

    a = np.asarray(a)
    b = np.asarray(b)
    return np.linalg.norm(a - b) <= prec * min(np.linalg.norm(a), np.linalg.norm(b))
