import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA device (GB300)')


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + '.npz')) as z:
        return {k: z[k] for k in z.files}


PLAN_CASES = ['plan_1d', 'plan_2d', 'plan_2d_odd', 'plan_3d', 'plan_3d_aniso', 'plan_2d_grid',
              'plan_2d_J8']


@pytest.fixture(scope='session')
def golden():
    return load_golden
