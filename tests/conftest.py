import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line('markers',
                            'gpu: needs a GB300 GPU and the built library')


@pytest.fixture(scope='session')
def golden():
    import numpy as np
    d = ROOT / 'tests' / 'golden'
    return {p.stem: dict(np.load(p)) for p in d.glob('*.npz')}
