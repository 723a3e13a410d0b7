import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, 'tests', 'golden')
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA device (GB300, sm_103a) and the built libsomgb.so')


def golden(name):
    with np.load(os.path.join(GOLDEN, f'{name}.npz'), allow_pickle=False) as f:
        return {k: f[k] for k in f.files}


@pytest.fixture(scope='session')
def oracle():
    from oracle import somref
    somref.lib()
    return somref


@pytest.fixture(scope='session')
def native():
    """The CUDA library, built if needed. GPU tests fail (they do not skip) when there is no device."""
    from decontamination_gb300 import build, _native
    build.build()
    _native.lib()
    return _native


@pytest.fixture(scope='session')
def cuda():
    import torch
    assert torch.cuda.is_available(), 'GPU tests need a CUDA device'
    major, minor = torch.cuda.get_device_capability()
    assert (major, minor) == (10, 3), f'expected an sm_103 device, found sm_{major}{minor}'
    return torch.device('cuda', 0)
