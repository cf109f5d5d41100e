import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, 'tests', 'golden')
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA device (GB300, sm_103a) and the built library')
    config.addinivalue_line('markers', 'slow: long-running case')


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + '.npz')) as d:
        return {k: d[k] for k in d.files}


@pytest.fixture
def golden():
    return load_golden


def grid_from(rec, prefix):
    from oracle.grids import RegularGrid
    return RegularGrid(rec[prefix + '_delta'], rec[prefix + '_dims'], rec[prefix + '_zero'])


def rel_err(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
