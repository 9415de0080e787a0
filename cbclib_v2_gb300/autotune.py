"""Autotuner of the render configuration (cbc_tuning): strategy, tile shape, threads
per CTA and lines per shared-memory chunk.

``tune`` times every candidate on the caller's data with CUDA events (on a scratch
copy of the frames) and keeps the fastest.  Results are cached per workload class:
device name, frame size, dtype, profile, overlap and a power-of-two bucket of the line
density (lines per megapixel), in memory and in a JSON file
(``$CBC_AUTOTUNE_CACHE``, default ``~/.cache/cbclib_v2_gb300/autotune.json``).
``draw_lines`` uses a cached choice for its workload class when there is one.
"""
import json
import math
import os
import threading
from typing import Dict, List, Optional, Tuple

import torch

from . import _native

__all__ = ['candidates', 'workload_key', 'lookup', 'tune', 'cache_path']

_lock = threading.Lock()
_mem: Dict[str, Tuple[int, ...]] = {}
_loaded = False


def cache_path() -> str:
    return os.environ.get('CBC_AUTOTUNE_CACHE',
                          os.path.join(os.path.expanduser('~'), '.cache', 'cbclib_v2_gb300',
                                       'autotune.json'))


def candidates() -> List[_native.Tuning]:
    T = _native.Tuning
    L, TI = _native.STRATEGY_LINES, _native.STRATEGY_TILES
    return [T(0, 0, 0, 0, L, 0),
            T(64, 64, 8, 256, TI, 0), T(64, 64, 16, 128, TI, 0), T(64, 32, 16, 128, TI, 0),
            T(32, 32, 16, 128, TI, 0), T(128, 64, 8, 256, TI, 0), T(128, 32, 16, 256, TI, 0)]


_names: Dict[int, str] = {}


def _device_name(device: Optional[torch.device]) -> str:
    if not torch.cuda.is_available():
        return 'cpu'
    idx = torch.cuda.current_device() if device is None or device.index is None else device.index
    name = _names.get(idx)
    if name is None:
        name = _names[idx] = torch.cuda.get_device_name(idx)
    return name


def workload_key(shape, dtype: torch.dtype, kernel: str, overlap: str, n_lines: int,
                 device: Optional[torch.device] = None) -> str:
    H, W = int(shape[-2]), int(shape[-1])
    F = math.prod(int(s) for s in shape[:-2])
    mpx = max(F * H * W / 1e6, 1e-6)
    bucket = int(math.floor(math.log2(max(n_lines / mpx, 1.0))))
    return f"{_device_name(device)}|{H}x{W}|{str(dtype).split('.')[-1]}|{kernel}|{overlap}|d{bucket}"


def _load():
    global _loaded
    if _loaded:
        return
    _loaded = True
    try:
        with open(cache_path()) as fh:
            for k, v in json.load(fh).items():
                _mem.setdefault(k, tuple(int(x) for x in v))
    except (OSError, ValueError):
        pass


def _save():
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + f'.{os.getpid()}.tmp'
        with open(tmp, 'w') as fh:
            json.dump({k: list(v) for k, v in _mem.items()}, fh, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def lookup(key: str) -> Optional[_native.Tuning]:
    with _lock:
        _load()
        v = _mem.get(key)
    return None if v is None else _native.Tuning(*v)


def has_entries() -> bool:
    """whether any workload class has a cached choice (lets callers skip the key)"""
    with _lock:
        _load()
        return bool(_mem)


def _time_call(fn, repeats: int) -> float:
    fn()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    for _ in range(repeats):
        fn()
    b.record(s)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / repeats


def tune(out: torch.Tensor, lines: torch.Tensor, idxs=None, max_val: float = 1.0,
         kernel: str = 'rectangular', overlap: str = 'sum', repeats: int = 3,
         frame_offsets: Optional[torch.Tensor] = None,
         store: bool = True) -> Tuple[_native.Tuning, Dict[str, float]]:
    """Time every candidate configuration on this data and return the fastest with all
    timings (ms per call).  ``out`` is not modified."""
    from . import ndimage
    k, ov = ndimage._check_names(kernel, overlap)
    scratch = out.detach().clone()
    timings = {}
    best, best_ms = None, float('inf')
    for t in candidates():
        if frame_offsets is not None:
            fn = lambda t=t: ndimage.draw_lines_csr(scratch, lines, frame_offsets, max_val,
                                                    kernel, overlap, tuning=t)
        else:
            fn = lambda t=t: ndimage._draw_lines_cuda(scratch, lines, idxs, max_val, k, ov,
                                                      tuning=t)
        ms = _time_call(fn, repeats)
        label = ('lines' if t.strategy == _native.STRATEGY_LINES else
                 f'tiles {t.tile_w}x{t.tile_h} t{t.threads} c{t.chunk_lines}')
        timings[label] = ms
        if ms < best_ms:
            best, best_ms = t, ms
    if store:
        key = workload_key(out.shape, out.dtype, kernel, overlap, lines.shape[0], out.device)
        with _lock:
            _load()
            _mem[key] = tuple(getattr(best, f) for f, _ in _native.Tuning._fields_)
            _save()
    return best, timings
