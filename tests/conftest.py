import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, 'tests', 'golden', 'draw_lines_golden.npz')


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: long-running test")


def load_golden():
    """{case name: {field: value}} of tests/golden/draw_lines_golden.npz"""
    z = np.load(GOLDEN)
    cases = {}
    for key in z.files:
        name, field = key.split('/')
        val = z[key]
        if val.dtype.kind == 'U':
            val = str(val)
        elif val.ndim == 0:
            val = val.item()
        cases.setdefault(name, {})[field] = val
    for c in cases.values():
        if 'out0' not in c:
            c['out0'] = np.zeros_like(c['result'])
    return cases


@pytest.fixture(scope='session')
def golden():
    return load_golden()


@pytest.fixture(scope='session')
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device('cuda')


@pytest.fixture(autouse=True)
def _seeded_torch():
    """every test starts from the same torch random state (CPU and CUDA generators)"""
    import torch
    torch.manual_seed(1234)
