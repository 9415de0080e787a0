"""The device module (reference README.md:50-65) and the host-side checks of the
public op; nothing here launches a kernel."""
import numpy as np
import pytest

from cbclib_v2_gb300 import device, draw_lines


def test_context_restores():
    before = device.get_device()
    with device.context('cpu'):
        assert device.get_device() == 'cpu'
    assert device.get_device() == before


def test_unknown_device():
    with pytest.raises(ValueError):
        device.set_device('tpu')
    with pytest.raises(ValueError):
        with device.context('metal'):
            pass


def test_cpu_device_has_no_fallback():
    out = np.zeros((8, 8), np.float32)
    lines = np.array([[1, 1, 6, 6, 1.0]], np.float32)
    with device.context('cpu'):
        with pytest.raises(RuntimeError, match='no CPU implementation'):
            draw_lines(out, lines)


@pytest.mark.parametrize("kw,exc", [(dict(kernel='box'), ValueError),
                                    (dict(overlap='min'), ValueError)])
def test_bad_names(kw, exc):
    with pytest.raises(exc):
        draw_lines(np.zeros((4, 4), np.float32), np.zeros((1, 5), np.float32), **kw)


def test_cuda_context_requires_gpu():
    if device.is_cuda_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError):
        device.set_device('cuda')
