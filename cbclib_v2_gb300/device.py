"""Device selection, the ``cbclib_v2.device`` contract documented in the reference's
README (README.md:50-65): ``is_cuda_available()``, ``set_device(name)`` and the
``context(name)`` manager that restores the previous device on exit.

Dispatch follows the reference's rule of deciding by the array type
(cbclib_v2/_src/functions.py:25-80): CUDA tensors always run on the GPU.  Host arrays
(NumPy, CPU tensors) run on the GPU, staged through device memory, while the device
is ``'cuda'`` (the default when a GPU is present).  This package has no CPU
implementation: with the device set to ``'cpu'`` host arrays raise ``RuntimeError``.
"""
import contextlib
import threading
from typing import Iterator, Optional

_NAMES = {'cuda': 'cuda', 'gpu': 'cuda', 'cpu': 'cpu'}
_state = threading.local()
_default: Optional[str] = None


def is_cuda_available() -> bool:
    """True when PyTorch sees a CUDA device."""
    import torch
    return bool(torch.cuda.is_available())


def _normalise(name: str) -> str:
    key = str(name).split(':')[0].lower()
    if key not in _NAMES:
        raise ValueError(f"Unknown device '{name}', expected 'cpu' or 'cuda'")
    return _NAMES[key]


def get_device() -> str:
    """The current device name, 'cuda' or 'cpu'."""
    cur = getattr(_state, 'device', None)
    if cur is not None:
        return cur
    if _default is not None:
        return _default
    return 'cuda' if is_cuda_available() else 'cpu'


def set_device(name: str) -> None:
    """Select the device for host arrays; applies to all threads without a context."""
    global _default
    dev = _normalise(name)
    if dev == 'cuda' and not is_cuda_available():
        raise RuntimeError("CUDA backend is not available on this machine")
    _default = dev
    _state.device = None


@contextlib.contextmanager
def context(name: str) -> Iterator[str]:
    """Run a block with ``name`` as the current device of this thread."""
    dev = _normalise(name)
    if dev == 'cuda' and not is_cuda_available():
        raise RuntimeError("CUDA backend is not available on this machine")
    prev = getattr(_state, 'device', None)
    _state.device = dev
    try:
        yield dev
    finally:
        _state.device = prev
