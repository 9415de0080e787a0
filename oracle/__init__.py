"""ORACLE — test infrastructure only (imported by tests/, ``__graft_entry__.smoke()`` and
the cpu_baseline / ``--impl reference`` legs of ``bench.py``; never by the product).

``draw_lines`` / ``accumulate_lines`` here run the plain-C restatement of the reference
CPU rasteriser (``cbc_oracle.c``, following cbclib_v2/_src/src/bresenham.{hpp,cpp}) on
NumPy arrays, with the reference's Python signature
(cbclib_v2/_src/functions.py:275-302 and :195-233) plus ``num_threads``.

``reference_module()`` returns the reference project's own compiled ``bresenham`` module
when ``oracle/build_ref.sh`` could build it (only where the reference checkout exists).
"""
import ctypes
import glob
import importlib.util
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
KERNELS = {'biweight': 0, 'gaussian': 1, 'parabolic': 2, 'rectangular': 3, 'triangular': 4}
OVERLAPS = {'sum': 0, 'max': 1}

_lib = None


def _load():
    global _lib
    if _lib is None:
        from . import build
        path = build.build_oracle()
        lib = ctypes.CDLL(path)
        p = ctypes.c_void_p
        i64 = ctypes.c_int64
        for sfx, real in (('f32', ctypes.c_float), ('f64', ctypes.c_double)):
            f = getattr(lib, f'cbc_oracle_draw_lines_{sfx}')
            f.argtypes = [p, i64, ctypes.c_int, p, p, i64, p, real, ctypes.c_int, ctypes.c_int,
                          ctypes.c_int]
            f.restype = ctypes.c_int
            f = getattr(lib, f'cbc_oracle_accumulate_lines_{sfx}')
            f.argtypes = [p, i64, ctypes.c_int, p, p, i64, p, p, i64, real, ctypes.c_int,
                          ctypes.c_int, ctypes.c_int, ctypes.c_int]
            f.restype = ctypes.c_int
            f = getattr(lib, f'cbc_oracle_profile_{sfx}')
            f.argtypes = [ctypes.c_int, real]
            f.restype = real
        lib.cbc_oracle_pixel_error_f32.argtypes = [ctypes.c_float] * 4
        lib.cbc_oracle_pixel_error_f32.restype = ctypes.c_float
        _lib = lib
    return _lib


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


def _raise(rc: int, what: str):
    if rc == 1:
        raise ValueError(f"{what}: invalid argument")
    if rc == 2:
        raise IndexError(f"{what}: index out of range")
    if rc:
        raise RuntimeError(f"{what}: error {rc}")


def _frames(out: np.ndarray, ndim: int):
    if out.ndim < ndim:
        raise ValueError("out has fewer dimensions than the lines")
    shape = np.asarray(out.shape[out.ndim - ndim:], dtype=np.int64)
    n_frames = int(np.prod(out.shape[:out.ndim - ndim], dtype=np.int64))
    return n_frames, shape


def draw_lines(out: np.ndarray, lines: np.ndarray, idxs: Optional[np.ndarray] = None,
               max_val: float = 1.0, kernel: str = 'rectangular', overlap: str = 'sum',
               num_threads: int = 1) -> np.ndarray:
    """Reference-semantics ``draw_lines`` on the CPU (mutates and returns ``out``)."""
    lib = _load()
    if out.dtype not in (np.float32, np.float64) or not out.flags.c_contiguous:
        raise ValueError("out must be a C-contiguous float32/float64 array")
    sfx = 'f32' if out.dtype == np.float32 else 'f64'
    L = lines.shape[-1]
    if L not in (5, 7):
        raise RuntimeError(f"Invalid lines size ({L})")
    ndim = (L - 1) // 2
    ln = np.ascontiguousarray(lines, dtype=out.dtype).reshape(-1, L)
    n_frames, shape = _frames(out, ndim)
    if kernel not in KERNELS:
        raise ValueError(f"kernel is missing for {kernel}")
    if overlap not in OVERLAPS:
        raise ValueError(f"Invalid overlap keyword: {overlap}")
    ix = None
    if idxs is not None:
        ix = np.ascontiguousarray(idxs, dtype=np.int64).ravel()
        if ix.size != ln.shape[0]:
            raise ValueError(f"idxs has an invalid size ({ix.size} != {ln.shape[0]})")
    rc = getattr(lib, f'cbc_oracle_draw_lines_{sfx}')(
        _ptr(out), n_frames, ndim, _ptr(shape), _ptr(ln), ln.shape[0],
        _ptr(ix) if ix is not None else None, max_val, KERNELS[kernel], OVERLAPS[overlap],
        int(num_threads))
    _raise(rc, 'draw_lines')
    return out


def accumulate_lines(out: np.ndarray, lines: np.ndarray, terms: np.ndarray, frames: np.ndarray,
                     max_val: float = 1.0, kernel: str = 'rectangular', in_overlap: str = 'sum',
                     out_overlap: str = 'sum', num_threads: int = 1) -> np.ndarray:
    """Reference-semantics ``accumulate_lines`` on the CPU (mutates and returns ``out``),
    terms shared out among ``num_threads`` threads as the reference does."""
    lib = _load()
    if out.dtype not in (np.float32, np.float64) or not out.flags.c_contiguous:
        raise ValueError("out must be a C-contiguous float32/float64 array")
    sfx = 'f32' if out.dtype == np.float32 else 'f64'
    L = lines.shape[-1]
    if L not in (5, 7):
        raise RuntimeError(f"Invalid lines size ({L})")
    ndim = (L - 1) // 2
    ln = np.ascontiguousarray(lines, dtype=out.dtype).reshape(-1, L)
    n_frames, shape = _frames(out, ndim)
    tm = np.ascontiguousarray(terms, dtype=np.int64).ravel()
    fr = np.ascontiguousarray(frames, dtype=np.int64).ravel()
    if tm.size != ln.shape[0]:
        raise ValueError("Term indices are incompatible with number of lines")
    if in_overlap not in OVERLAPS or out_overlap not in OVERLAPS:
        raise ValueError(f"Invalid in_overlap and out_overlap keywords: {in_overlap} and "
                         f"{out_overlap}")
    rc = getattr(lib, f'cbc_oracle_accumulate_lines_{sfx}')(
        _ptr(out), n_frames, ndim, _ptr(shape), _ptr(ln), ln.shape[0], _ptr(tm), _ptr(fr),
        fr.size, max_val, KERNELS[kernel], OVERLAPS[in_overlap], OVERLAPS[out_overlap],
        int(num_threads))
    _raise(rc, 'accumulate_lines')
    return out


def profile(kernel: str, x: float, dtype=np.float32) -> float:
    """One profile value K(x) with the reference's float/double arithmetic."""
    lib = _load()
    sfx = 'f32' if np.dtype(dtype) == np.float32 else 'f64'
    return getattr(lib, f'cbc_oracle_profile_{sfx}')(KERNELS[kernel], x)


def pixel_error_f32(te: float, ne: float, length: float, width: float) -> float:
    """BresenhamPlotter::error of a 2-D position from its tangent/normal errors (f32)."""
    return _load().cbc_oracle_pixel_error_f32(te, ne, length, width)


def reference_module():
    """The reference project's own compiled ``bresenham`` module, or None."""
    cands = glob.glob(os.path.join(HERE, '_ref', 'bresenham*.so'))
    if not cands:
        return None
    spec = importlib.util.spec_from_file_location('bresenham', cands[0])
    mod = importlib.util.module_from_spec(spec)
    try:
        spec.loader.exec_module(mod)
    except ImportError:
        return None
    return mod
