import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the compiled libsnch_gb300.so")


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def load_golden(name):
    with np.load(os.path.join(GOLDEN_DIR, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def d1_tainted(nodes, d1):
    """Nodes whose cone depends on a cone merge the reference leaves undefined
    (cone.cuh:454-458): the flagged nodes and all their ancestors."""
    taint = d1.astype(bool).copy()
    for n in np.nonzero(d1)[0]:
        p = nodes[n, 0]
        while p != 0xFFFFFFFF:
            taint[p] = True
            p = nodes[p, 0]
    return taint


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle
