"""Drop-in ``cbclib_v2.ndimage.draw_lines`` on the GB300 kernels.

Same signature, argument meaning and error behaviour as the reference's public op
(cbclib_v2/_src/functions.py:275-302, pybind11 binding bresenham.cpp:329-330):
``out`` is updated in place and returned.  Results are those of the reference CPU
path bit for bit (max overlap, and sum apart from the order in which several lines'
contributions to one pixel are added).
"""
import contextlib
import math
import threading
from typing import Iterator, Optional, Tuple

import numpy as np
import torch

from . import _native
from . import device as _device

__all__ = ['draw_lines', 'draw_lines_csr', 'accumulate_lines', 'Workspace', 'tuning',
           'release_scratch', 'deferred_errors']

_tls = threading.local()


@contextlib.contextmanager
def tuning(**fields) -> Iterator[_native.Tuning]:
    """Force render settings (cbc_tuning fields: tile_w, tile_h, chunk_lines, threads,
    strategy) for the draw_lines calls of this thread inside the block."""
    t = _native.Tuning()
    for k, v in fields.items():
        if not hasattr(t, k):
            raise AttributeError(f"cbc_tuning has no field {k!r}")
        setattr(t, k, int(v))
    prev = getattr(_tls, 'tuning', None)
    _tls.tuning = t
    try:
        yield t
    finally:
        _tls.tuning = prev


class Workspace:
    """Device scratch of one (device, stream, thread): grows on demand, reused by calls.

    Layout and size come from ``cbc_draw_lines_workspace_size``; the pair capacity grows
    when a call reports that its (line, tile) pairs did not fit."""

    def __init__(self, dev: torch.device):
        self.device = dev
        self.buffer: Optional[torch.Tensor] = None
        self.capacity = 0
        self.ck_capacity = 0
        self.last_status: Optional[_native.Status] = None
        self.size_key = None             # arguments and result of the last size query
        self.size_bytes = 0

    def ensure(self, nbytes: int) -> torch.Tensor:
        if self.buffer is None or self.buffer.numel() < nbytes:
            self.buffer = torch.empty(int(nbytes * 1.1) + 4096, dtype=torch.uint8,
                                      device=self.device)
        return self.buffer


_ws_lock = threading.Lock()
_workspaces = {}


def _workspace(dev: torch.device, stream: torch.cuda.Stream) -> Workspace:
    return _workspace_raw(dev, stream.cuda_stream)


def _workspace_raw(dev: torch.device, stream: int) -> Workspace:
    key = (dev.index, stream, threading.get_ident())
    ws = _workspaces.get(key)           # dict reads are atomic; creation takes the lock
    if ws is None:
        with _ws_lock:
            ws = _workspaces.setdefault(key, Workspace(dev))
    return ws


def _check_names(kernel: str, overlap: str) -> Tuple[int, int]:
    if kernel not in _native.KERNELS:
        raise ValueError(f"kernel is missing for {kernel}")
    if overlap not in _native.OVERLAPS:
        raise ValueError(f"Invalid overlap keyword: {overlap}")
    return _native.KERNELS[kernel], _native.OVERLAPS[overlap]


def _as_device_lines(lines, dev: torch.device, dtype: torch.dtype) -> torch.Tensor:
    t = torch.as_tensor(lines)
    if t.ndim < 1:
        raise ValueError("lines must have at least one dimension")
    L = t.shape[-1]
    if L not in (5, 7):
        raise RuntimeError(f"Invalid lines size ({L}) at axis {t.ndim - 1}")
    return t.to(device=dev, dtype=dtype).reshape(-1, L).contiguous()


def _volumes_of(out: torch.Tensor):
    """(F, D, H, W) of an output for 3-D lines"""
    if out.dtype not in (torch.float32, torch.float64):
        raise TypeError(f"out must be float32 or float64, got {out.dtype}")
    if out.dim() < 3:
        raise ValueError(f"Output array dimensions ({out.dim()}) do not match the line size (7)")
    D, H, W = (int(s) for s in out.shape[-3:])
    return math.prod(int(s) for s in out.shape[:-3]), D, H, W


def _columns3(ln: torch.Tensor, extent: int) -> int:
    """An upper estimate of the long-axis columns of (N, 7) 3-D lines in volumes whose
    largest side is ``extent``: the 3-D renders keep one walk checkpoint per column."""
    span = (ln[:, 3:6] - ln[:, 0:3]).abs().amax(dim=1) + 2 * ln[:, 6].clamp(min=0).ceil() + 3
    span = torch.nan_to_num(span, nan=0.0, posinf=float(extent), neginf=0.0)
    return int(span.clamp(max=float(extent)).sum().item())


def _run3(call, size, dev: torch.device, kind: str, n_frames: int, n_lines: int,
          table: bool = False, on_status=None, columns=None) -> None:
    """Run a 3-D library call ``call(buf, ck_capacity, table_capacity, stream)`` with
    this thread's workspace, raise the status' errors and retry with more room when the
    call reports that its checkpoints or (``table``: mixed-overlap accumulate) its
    workspace table did not fit.  ``columns()`` estimates the checkpoints the call
    needs; it runs (one synchronisation) only when the workspace's are fewer than the
    default."""
    lib = _native.lib()
    with torch.cuda.device(dev):
        stream = torch.cuda.current_stream(dev)
        key = (kind, dev.index, stream.cuda_stream, threading.get_ident())
        with _ws_lock:
            ws = _workspaces.setdefault(key, Workspace(dev))
        ck_capacity = max(ws.ck_capacity, 16 * n_lines + 1024)
        if columns is not None and ws.ck_capacity < ck_capacity:
            ck_capacity = max(ck_capacity, int(columns() * 1.25) + 1024)
        table_cap = ws.capacity if table else 0
        for _ in range(6):
            buf = ws.ensure(size(ck_capacity, table_cap))
            rc = call(buf, ck_capacity, table_cap, stream.cuda_stream)
            if rc:
                _raise_rc(rc)
            st = _native.Status()
            if lib.cbc_read_status(buf.data_ptr(), st, stream.cuda_stream):
                _raise_rc(_native.CBC_ERR_CUDA)
            ws.last_status = st
            if on_status is not None:
                on_status(st)
            _raise_status(st, n_frames)
            if not st.has(_native.CBC_ERR_CAPACITY):
                ws.ck_capacity = ck_capacity
                ws.capacity = table_cap
                return
            ck_capacity = max(ck_capacity, int(st.checkpoints_needed * 1.25) + 1024)
            if table:
                table_cap = max(table_cap, int(st.pairs_needed))
            if ck_capacity > 2**31 - 1:
                raise MemoryError("too many walk checkpoints for one call")
    raise RuntimeError("workspace capacity did not converge")


def _draw_lines3d_cuda(out: torch.Tensor, ln: torch.Tensor, idxs, max_val: float, kernel: int,
                       overlap: int) -> torch.Tensor:
    F, D, H, W = _volumes_of(out)
    n_lines = ln.shape[0]
    ix = _as_device_idxs(idxs, n_lines, out.device)
    if ix is None and n_lines and F != 1 and F != n_lines:
        raise ValueError(f"idxs has an incompatible size ({n_lines} != {F})")
    work = out if out.is_contiguous() else out.contiguous()
    elem = 4 if out.dtype == torch.float32 else 8
    lib = _native.lib()
    fn = lib.cbc_draw_lines_3d_f32 if elem == 4 else lib.cbc_draw_lines_3d_f64
    _run3(lambda buf, ck, _t, stream: fn(
              work.data_ptr(), F, D, H, W, ln.data_ptr(), n_lines,
              None if ix is None else ix.data_ptr(), 0 if ix is None else ix.element_size(),
              max_val, kernel, overlap, buf.data_ptr(), buf.numel(), ck, stream),
          lambda ck, _t: lib.cbc_draw_lines_3d_workspace_size(n_lines, ck, elem),
          out.device, 'draw3d', F, n_lines, columns=lambda: _columns3(ln, max(D, H, W)))
    if work is not out:
        out.copy_(work)
    return out


def _as_device_idxs(idxs, n_lines: int, dev: torch.device) -> Optional[torch.Tensor]:
    if idxs is None:
        return None
    t = torch.as_tensor(idxs)
    if t.is_floating_point() or t.is_complex() or t.dtype == torch.bool:
        raise TypeError("idxs must be an integer array")
    t = t.reshape(-1)
    if t.numel() != n_lines:
        raise ValueError(f"idxs has an invalid size ({t.numel()} != {n_lines})")
    if t.dtype not in (torch.int32, torch.int64):
        t = t.to(torch.int64)
    return t.to(device=dev).contiguous()


def _raise_status(st: _native.Status, n_frames: int):
    if st.has(_native.CBC_ERR_CUDA):
        raise RuntimeError("a device-side wait for an asynchronous copy gave up; the "
                           "result of the call is incomplete")
    if st.has(_native.CBC_ERR_INDEX):
        raise IndexError(f"idxs range ({st.idx_min}, {st.idx_max}) is outside of "
                         f"(0, {n_frames})")
    if st.has(_native.CBC_ERR_RANGE):
        raise ValueError(f"line {st.bad_line}: its walk is longer than {_native.MAX_WALK} "
                         "pixels or its coordinates exceed 2^30")


def _raise_rc(rc: int):
    msg = _native.last_error()
    if rc == _native.CBC_ERR_INVALID:
        raise ValueError(msg)
    raise RuntimeError(f"cbc_draw_lines failed ({rc}): {msg}")


def _resolve_tuning(tuning, out: torch.Tensor, n_lines: int, kernel: int, overlap: int):
    """forced tuning > this thread's `tuning(...)` block > autotuned choice > default"""
    if tuning is None:
        tuning = getattr(_tls, 'tuning', None)
    if tuning is None:
        from . import autotune
        if autotune.has_entries():
            tuning = autotune.lookup(autotune.workload_key(
                out.shape, out.dtype, _KERNEL_NAMES[kernel], _OVERLAP_NAMES[overlap], n_lines,
                out.device))
    return tuning


_KERNEL_NAMES = {v: k for k, v in _native.KERNELS.items()}
_OVERLAP_NAMES = {v: k for k, v in _native.OVERLAPS.items()}


def _current_stream(dev: torch.device) -> int:
    """raw handle of the current stream of `dev`"""
    raw = getattr(torch._C, '_cuda_getCurrentRawStream', None)
    if raw is not None:
        return raw(dev.index)
    return torch.cuda.current_stream(dev).cuda_stream


class _on_current_device:
    """`with torch.cuda.device(dev)` that costs nothing when `dev` is already current"""
    def __init__(self, dev: torch.device):
        self.dev = dev
        self.ctx = None

    def __enter__(self):
        if self.dev.index != torch.cuda.current_device():
            self.ctx = torch.cuda.device(self.dev)
            self.ctx.__enter__()

    def __exit__(self, *exc):
        if self.ctx is not None:
            self.ctx.__exit__(*exc)


class _Deferred:
    """the calls of one deferred_errors() block: a page-locked copy of each call's
    device status and a function that runs the call again with room to spare"""

    def __init__(self):
        self.pending = []                # (status bytes, rerun, n_frames, device)

    def finish(self) -> None:
        lib = _native.lib()
        for dev in {d for _, _, _, d in self.pending}:
            torch.cuda.synchronize(dev)
        pending, self.pending = self.pending, []
        for buf, rerun, n_frames, _ in pending:
            st = _native.Status()
            lib.cbc_decode_status(buf.data_ptr(), st)
            _raise_status(st, n_frames)
            if st.has(_native.CBC_ERR_CAPACITY):
                rerun()                  # it drew nothing: run it again, checked


@contextlib.contextmanager
def deferred_errors() -> Iterator[None]:
    """Inside the block, draw_lines and draw_lines_csr calls on contiguous CUDA frames
    return without waiting for the GPU: each call's device status (index and range
    errors, and whether its walks fitted the workspace) is copied to page-locked host
    memory asynchronously and all of them are checked when the block exits, after
    waiting for the devices.  Back-to-back calls then queue on the stream while the
    host prepares the next one.  On exit the first error raises (IndexError,
    ValueError), as the call itself would have; a call that drew nothing because its
    walks needed more room than the workspace held is run again then, in the order of
    the block (overlaps combine in any order; float sums may differ in the last bits).
    Host frames, other entry points and calls outside the block check as usual."""
    prev = getattr(_tls, 'deferred', None)
    d = _Deferred()
    _tls.deferred = d
    try:
        yield
    finally:
        _tls.deferred = prev
    d.finish()


def _run_with_workspace(call, dev: torch.device, F: int, H: int, W: int, n_lines: int,
                        elem: int, tuning, size_fn=None, deferrable: bool = False) -> None:
    """Run `call(buf, capacity, ck_capacity, tref, stream)` with this thread's
    workspace, read the status, raise the reference's errors and repeat with a larger
    workspace when the call reports that its pairs or checkpoints did not fit.
    ``size_fn(F, H, W, n_lines, capacity, ck_capacity)`` sizes the workspace of calls
    whose workspace starts with a draw_lines one (default: the draw_lines size).  With
    ``deferrable`` inside a deferred_errors() block the status is only copied
    asynchronously (checked when the block exits)."""
    lib = _native.lib()
    deferred = getattr(_tls, 'deferred', None) if deferrable else None
    with _on_current_device(dev):
        stream = _current_stream(dev)
        ws = _workspace_raw(dev, stream)
        capacity = max(ws.capacity, 4 * n_lines + 1024)
        ck_capacity = max(ws.ck_capacity, 16 * n_lines + 1024)
        tref = None if tuning is None else ctypes_pointer(tuning)
        for _ in range(4):
            size_key = (size_fn, F, H, W, n_lines, capacity, ck_capacity, elem,
                        None if tuning is None else tuple(getattr(tuning, f) for f, _ in
                                                          _native.Tuning._fields_))
            if ws.size_key == size_key:
                nbytes = ws.size_bytes
            else:
                nbytes = (size_fn(F, H, W, n_lines, capacity, ck_capacity) if size_fn else
                          lib.cbc_draw_lines_workspace_size(F, H, W, n_lines, capacity,
                                                            ck_capacity, elem, tref))
                if nbytes == 0:
                    raise ValueError(_native.last_error() or "invalid sizes or tuning")
                ws.size_key, ws.size_bytes = size_key, nbytes
            buf = ws.ensure(nbytes)
            rc = call(buf, capacity, ck_capacity, tref, stream)
            if rc:
                _raise_rc(rc)
            if deferred is not None:
                slot = torch.empty(int(lib.cbc_status_bytes()), dtype=torch.uint8,
                                   pin_memory=True)
                rc = lib.cbc_copy_status_async(buf.data_ptr(), slot.data_ptr(), stream)
                if rc:
                    _raise_rc(rc)
                ws.capacity, ws.ck_capacity = capacity, ck_capacity
                deferred.pending.append((slot, lambda: _run_with_workspace(
                    call, dev, F, H, W, n_lines, elem, tuning, size_fn), F, dev))
                return
            st = _native.Status()
            rc = lib.cbc_read_status(buf.data_ptr(), st, stream)
            if rc:
                _raise_rc(rc)
            ws.last_status = st
            _raise_status(st, F)
            if not st.has(_native.CBC_ERR_CAPACITY):
                ws.capacity = capacity
                ws.ck_capacity = ck_capacity
                return
            capacity = max(capacity, int(st.pairs_needed * 1.25) + 1024)
            ck_capacity = max(ck_capacity, int(st.checkpoints_needed * 1.25) + 1024)
            if capacity > 2**31 - 1 or ck_capacity > 2**31 - 1:
                raise MemoryError("too many (line, tile) pairs or walk checkpoints for one call")
    raise RuntimeError("workspace capacity did not converge")


def last_status(dev=None) -> Optional[_native.Status]:
    """Status of the calling thread's last draw_lines call on the current stream of
    `dev` (None before the first call): error flags, the render strategy that ran and
    the pair / checkpoint counts."""
    dev = torch.device('cuda', torch.cuda.current_device()) if dev is None else torch.device(dev)
    return _workspace(dev, torch.cuda.current_stream(dev)).last_status


def _frames_of(out: torch.Tensor):
    if out.dtype not in (torch.float32, torch.float64):
        raise TypeError(f"out must be float32 or float64, got {out.dtype}")
    if out.dim() < 2:
        raise ValueError("Output array has insufficient number of dimensions")
    H, W = int(out.shape[-2]), int(out.shape[-1])
    F = math.prod(int(s) for s in out.shape[:-2])
    return F, H, W


def _draw_lines_cuda(out: torch.Tensor, lines, idxs, max_val: float, kernel: int,
                     overlap: int, tuning: Optional[_native.Tuning] = None) -> torch.Tensor:
    ln = _as_device_lines(lines, out.device, out.dtype)
    if ln.shape[1] == 7:
        return _draw_lines3d_cuda(out, ln, idxs, max_val, kernel, overlap)
    F, H, W = _frames_of(out)
    dev = out.device
    n_lines = ln.shape[0]
    ix = _as_device_idxs(idxs, n_lines, dev)
    if ix is None and n_lines and F != 1 and F != n_lines:
        raise ValueError(f"idxs has an incompatible size ({n_lines} != {F})")
    tuning = _resolve_tuning(tuning, out, n_lines, kernel, overlap)
    work = out if out.is_contiguous() else out.contiguous()
    elem = 4 if out.dtype == torch.float32 else 8
    lib = _native.lib()
    fn = lib.cbc_draw_lines_f32 if elem == 4 else lib.cbc_draw_lines_f64

    def call(buf, capacity, ck_capacity, tref, stream):
        return fn(work.data_ptr(), F, H, W, ln.data_ptr(), n_lines,
                  None if ix is None else ix.data_ptr(), 0 if ix is None else ix.element_size(),
                  max_val, kernel, overlap, buf.data_ptr(), buf.numel(), capacity, ck_capacity,
                  tref, stream)

    _run_with_workspace(call, dev, F, H, W, n_lines, elem, tuning, deferrable=work is out)
    if work is not out:
        out.copy_(work)
    return out


_packed: dict = {}


def _packed_scratch(dev: torch.device, n: int) -> torch.Tensor:
    """this thread's zeroed uint64 scratch of at least n values on the current stream of
    `dev` (the library leaves it zero after every call)"""
    key = (dev.index, _current_stream(dev), threading.get_ident())
    buf = _packed.get(key)
    if buf is None or buf.numel() < n:
        buf = _packed[key] = torch.zeros(n, dtype=torch.int64, device=dev)
    return buf


def draw_lines_max_winner(out: torch.Tensor, lines, idxs=None, max_val: float = 1.0,
                          kernel: str = 'rectangular',
                          winner: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Max-overlap draw_lines into float32 CUDA frames that start at zero (``out`` is
    overwritten) and the winner of every pixel: the line whose value the pixel holds
    (the smallest index among equal values, as sequential std::max keeps), or
    0x7f7f7f7f where no line raised the pixel above zero.  Returns ``winner`` (int32,
    the frames' shape; allocated when not given)."""
    if not (isinstance(out, torch.Tensor) and out.is_cuda and out.dtype == torch.float32):
        raise TypeError("out must be a float32 CUDA tensor")
    if winner is None:
        winner = torch.empty(out.shape, dtype=torch.int32, device=out.device)
    elif not (isinstance(winner, torch.Tensor) and winner.dtype == torch.int32 and
              winner.is_contiguous() and winner.numel() == out.numel() and
              winner.device == out.device):
        raise ValueError("winner must be a contiguous int32 tensor with one entry per pixel "
                         "of out, on out's device")
    work = out if out.is_contiguous() else torch.empty(out.shape, dtype=out.dtype,
                                                       device=out.device)
    _max_winner(work, winner, out.shape, out.device, lines, idxs, max_val, kernel)
    if work is not out:
        out.copy_(work)
    return winner


def _max_winner(out: Optional[torch.Tensor], winner: Optional[torch.Tensor], shape, dev,
                lines, idxs, max_val: float, kernel: str) -> torch.Tensor:
    """cbc_draw_lines_max_winner_f32 with this thread's packed scratch; with out and
    winner None the scratch is returned holding the (value, winner) pairs and the
    caller zeroes it after use"""
    k, _ = _check_names(kernel, 'max')
    H, W = int(shape[-2]), int(shape[-1])
    F = math.prod(int(s) for s in shape[:-2])
    ln = _as_device_lines(lines, dev, torch.float32)
    if ln.shape[1] != 5:
        raise ValueError("draw_lines_max_winner takes 2-D lines (N, 5)")
    n_lines = ln.shape[0]
    ix = _as_device_idxs(idxs, n_lines, dev)
    if ix is None and n_lines and F != 1 and F != n_lines:
        raise ValueError(f"idxs has an incompatible size ({n_lines} != {F})")
    packed = _packed_scratch(dev, F * H * W)
    lib = _native.lib()
    t = _native.Tuning()
    t.strategy = _native.STRATEGY_LINES

    def call(buf, capacity, ck_capacity, tref, stream):
        return lib.cbc_draw_lines_max_winner_f32(
            None if out is None else out.data_ptr(), None if winner is None else winner.data_ptr(),
            packed.data_ptr(), F, H, W, ln.data_ptr(),
            n_lines, None if ix is None else ix.data_ptr(),
            0 if ix is None else ix.element_size(), max_val, k, buf.data_ptr(), buf.numel(),
            capacity, ck_capacity, stream)

    _run_with_workspace(call, dev, F, H, W, n_lines, 4, t)
    return packed


def draw_lines_csr(out: torch.Tensor, lines, frame_offsets, max_val: float = 1.0,
                   kernel: str = 'rectangular', overlap: str = 'sum',
                   tuning: Optional[_native.Tuning] = None) -> torch.Tensor:
    """draw_lines for a ragged stack whose lines are grouped by frame: frame f owns
    lines[frame_offsets[f]:frame_offsets[f + 1]] (int64 CSR offsets, F + 1 entries).
    ``out`` is a CUDA tensor (..., H, W) updated in place."""
    k, ov = _check_names(kernel, overlap)
    F, H, W = _frames_of(out)
    dev = out.device
    ln = _as_device_lines(lines, dev, out.dtype)
    if ln.shape[1] != 5:
        raise ValueError("draw_lines_csr takes 2-D lines (N, 5)")
    n_lines = ln.shape[0]
    offs = torch.as_tensor(frame_offsets).to(device=dev, dtype=torch.int64).reshape(-1)
    if offs.numel() != F + 1:
        raise ValueError(f"frame_offsets has {offs.numel()} entries, expected {F + 1}")
    offs = offs.contiguous()
    tuning = _resolve_tuning(tuning, out, n_lines, k, ov)
    work = out if out.is_contiguous() else out.contiguous()
    elem = 4 if out.dtype == torch.float32 else 8
    lib = _native.lib()
    fn = lib.cbc_draw_lines_csr_f32 if elem == 4 else lib.cbc_draw_lines_csr_f64

    def call(buf, capacity, ck_capacity, tref, stream):
        return fn(work.data_ptr(), F, H, W, ln.data_ptr(), n_lines, offs.data_ptr(), max_val, k,
                  ov, buf.data_ptr(), buf.numel(), capacity, ck_capacity, tref, stream)

    _run_with_workspace(call, dev, F, H, W, n_lines, elem, tuning, deferrable=work is out)
    if work is not out:
        out.copy_(work)
    return out


def ctypes_pointer(t: _native.Tuning):
    import ctypes
    return ctypes.pointer(t)


def draw_lines(out, lines, idxs=None, max_val: float = 1.0, kernel: str = 'rectangular',
               overlap: str = 'sum'):
    """Draw thick lines with variable thickness and antialiasing into ``out``.

    Args:
        out: Output frames (..., H, W), float32 or float64.  A CUDA tensor (or any
            ``__cuda_array_interface__`` array) is updated in place on its device; a
            host array (NumPy, CPU tensor) is staged through the GPU and updated in
            place while the current device is 'cuda'.
        lines: (N, 5) rows [x0, y0, x1, y1, width], xy order.
        idxs: frame index of each line into the flattened leading dims of ``out``;
            None draws every line into frame 0 (single frame) or line i into frame i.
        max_val: peak value of a line's profile.
        kernel: 'biweight', 'gaussian', 'parabolic', 'rectangular' or 'triangular'.
        overlap: 'sum' or 'max' combination of overlapping lines.

    Returns:
        ``out``.
    """
    k, ov = _check_names(kernel, overlap)
    host = _host_tensor(out)
    if host is not None and _draw_lines_staged(host, lines, idxs, max_val, k, ov):
        return out
    return _on_device(out, 'draw_lines',
                      lambda dev_out: _draw_lines_cuda(dev_out, lines, idxs, max_val, k, ov))


def _host_tensor(out) -> Optional[torch.Tensor]:
    """a CPU tensor sharing the memory of a host array that the library may update in
    place (a CPU tensor, or a writable, aligned, C-contiguous NumPy array), else None"""
    if isinstance(out, torch.Tensor):
        return None if out.is_cuda else out
    if isinstance(out, np.ndarray) and out.flags.c_contiguous and out.flags.writeable and \
            out.flags.aligned and out.dtype in (np.float32, np.float64):
        return torch.from_numpy(out)
    return None


# device scratch frames of the host-frame path, per (device, stream, host thread),
# least recently used first; at most MAX_HOST_SCRATCH are kept (release_scratch()
# drops them all)
MAX_HOST_SCRATCH = 4
_host_scratch: dict = {}
_host_scratch_lock = threading.Lock()


def release_scratch() -> None:
    """Drop the library's cached device buffers of this process (workspaces, the
    host-frame scratch frames and the packed max scratch); later calls allocate them
    again.  Waits for the current devices' work first."""
    if torch.cuda.is_available():
        torch.cuda.synchronize()
    with _host_scratch_lock:
        _host_scratch.clear()
    with _ws_lock:
        _workspaces.clear()
    _packed.clear()


def _draw_lines_staged(host: torch.Tensor, lines, idxs, max_val: float, kernel: int,
                       overlap: int) -> bool:
    """draw_lines on host frames of 2-D lines without copying the frames: the kernels
    draw into a device scratch holding the overlap's identity and combine the drawn
    pixels into the host frames in place (cbc_draw_lines_host_*), through the device
    mapping of page-locked memory, or directly where the device reads and writes
    pageable memory coherently (NVLink-C2C systems; NumPy arrays included).  The
    scratch (one per device, stream and host thread) is left at the identity after
    every call; it is filled again only when the overlap, the dtype or the size
    changes.  Returns False when the frames do not qualify (memory the device cannot
    address, non-contiguous, 3-D lines or no device)."""
    if not (host.is_contiguous() and host.dim() >= 2 and host.numel() > 0 and
            host.dtype in (torch.float32, torch.float64)):
        return False
    if _device.get_device() != 'cuda':
        return False
    t = torch.as_tensor(lines)
    if t.ndim < 1 or t.shape[-1] != 5:
        return False
    F, H, W = _frames_of(host)
    dev = torch.device('cuda', torch.cuda.current_device())
    with _on_current_device(dev):
        if _native.host_access(host.data_ptr()) == _native.HOST_NONE:
            return False
        # lines and indices in host memory the device reads are read in place (the
        # kernels read each line once); others are copied to the device
        ln = _host_readable(t.reshape(-1, 5) if t.is_contiguous() else None, host.dtype)
        if ln is None:
            ln = _as_device_lines(t, dev, host.dtype)
        n = ln.shape[0]
        ix = None
        if idxs is not None:
            ti = torch.as_tensor(idxs)
            if ti.dtype in (torch.int32, torch.int64) and ti.numel() == n and ti.is_contiguous():
                ix = _host_readable(ti.reshape(-1), ti.dtype)
            if ix is None:
                ix = _as_device_idxs(idxs, n, dev)
    if ix is None and n and F != 1 and F != n:
        raise ValueError(f"idxs has an incompatible size ({n} != {F})")
    elem = 4 if host.dtype == torch.float32 else 8
    lib = _native.lib()
    fn = lib.cbc_draw_lines_host_f32 if elem == 4 else lib.cbc_draw_lines_host_f64
    tuning = getattr(_tls, 'tuning', None)
    with _on_current_device(dev):
        stream = _current_stream(dev)
        key = (dev.index, stream, threading.get_ident())
        tag = (overlap, host.dtype)
        with _host_scratch_lock:
            entry = _host_scratch.pop(key, None)
            if entry is None or entry[0].numel() < F * H * W or entry[0].dtype != host.dtype:
                entry = None
                while len(_host_scratch) >= MAX_HOST_SCRATCH:
                    _host_scratch.pop(next(iter(_host_scratch)))
            else:
                _host_scratch[key] = entry           # most recently used last
        if entry is None:
            # [buffer, overlap and dtype of its identity, elements holding that identity]
            entry = [torch.empty(F * H * W, dtype=host.dtype, device=dev), None, 0]
            with _host_scratch_lock:
                _host_scratch[key] = entry
        scratch = entry[0]
        # a call over more elements than the identity covers (a smaller stack with
        # another overlap came in between) fills its whole range again
        state = {'fill': int(entry[1] != tag or entry[2] < F * H * W)}

        def call(buf, capacity, ck_capacity, tref, stream):
            rc = fn(host.data_ptr(), F, H, W, ln.data_ptr(), n,
                    None if ix is None else ix.data_ptr(), 0 if ix is None else ix.element_size(),
                    max_val, kernel, overlap, scratch.data_ptr(), state['fill'], buf.data_ptr(),
                    buf.numel(), capacity, ck_capacity, tref, stream)
            if rc == 0:
                if state['fill']:
                    entry[2] = F * H * W
                state['fill'] = 0      # the scratch is at the identity from here on
                entry[1] = tag
            return rc

        entry[1] = None                # unknown until the call has run
        _run_with_workspace(call, dev, F, H, W, n, elem, tuning)
    return True


def _host_readable(t: Optional[torch.Tensor], dtype: torch.dtype) -> Optional[torch.Tensor]:
    """`t` itself when it is a contiguous, non-empty CPU tensor of `dtype` in pageable
    host memory that the current device reads at its own address (cbc_host_access,
    NVLink-C2C systems), else None (page-locked memory is copied: that is one DMA)"""
    if t is None or t.is_cuda or t.dtype != dtype or t.numel() == 0 or not t.is_contiguous():
        return None
    return t if _native.host_access(t.data_ptr()) == _native.HOST_PAGEABLE else None


def _on_device(out, name: str, run):
    """Run ``run(cuda_tensor)`` on ``out``: CUDA tensors and ``__cuda_array_interface__``
    arrays in place; host arrays (NumPy, CPU tensors) staged through the GPU and written
    back, while the current device is 'cuda'.  Returns ``out``."""
    if isinstance(out, torch.Tensor):
        if out.is_cuda:
            run(out)
            return out
        host = out
    elif hasattr(out, '__cuda_array_interface__'):
        run(torch.as_tensor(out, device='cuda'))
        return out
    else:
        host = out
    if _device.get_device() != 'cuda':
        raise RuntimeError(f"cbclib_v2_gb300 has no CPU implementation of {name}: select "
                           "the 'cuda' device or pass CUDA arrays")
    if isinstance(host, torch.Tensor):
        if host.dtype not in (torch.float32, torch.float64):
            raise TypeError(f"out must be float32 or float64, got {host.dtype}")
        dev_out = host.to('cuda')
        run(dev_out)
        host.copy_(dev_out)
        return out
    if not isinstance(host, np.ndarray):
        raise TypeError(f"unsupported output array type {type(out)}")
    if host.dtype not in (np.float32, np.float64):
        raise TypeError(f"out must be float32 or float64, got {host.dtype}")
    dev_out = torch.from_numpy(np.ascontiguousarray(host)).to('cuda')
    run(dev_out)
    if host.flags.c_contiguous and host.flags.writeable:
        torch.from_numpy(host).copy_(dev_out)
    else:
        np.copyto(host, dev_out.cpu().numpy())
    return out


def _as_device_ints(a, name: str, dev: torch.device) -> torch.Tensor:
    t = torch.as_tensor(a)
    if t.is_floating_point() or t.is_complex() or t.dtype == torch.bool:
        raise TypeError(f"{name} must be an integer array")
    t = t.reshape(-1)
    if t.dtype not in (torch.int32, torch.int64):
        t = t.to(torch.int64)
    return t.to(device=dev).contiguous()


def _accumulate_lines_cuda(out: torch.Tensor, lines, terms, frames, max_val: float, kernel: int,
                           in_ov: int, out_ov: int) -> torch.Tensor:
    dev = out.device
    ln = _as_device_lines(lines, dev, out.dtype)
    if ln.shape[1] == 7:
        return _accumulate_lines3d_cuda(out, ln, terms, frames, max_val, kernel, in_ov, out_ov)
    F, H, W = _frames_of(out)
    n_lines = ln.shape[0]
    tm = _as_device_ints(terms, 'terms', dev)
    if tm.numel() != n_lines:
        raise ValueError(f"Term indices ({tm.numel()}) is incompatible with number of lines "
                         f"({n_lines})")
    fr = _as_device_ints(frames, 'frames', dev)
    n_terms = fr.numel()
    work = out if out.is_contiguous() else out.contiguous()
    elem = 4 if out.dtype == torch.float32 else 8
    lib = _native.lib()
    fn = lib.cbc_accumulate_lines_f32 if elem == 4 else lib.cbc_accumulate_lines_f64
    table = in_ov != out_ov
    with torch.cuda.device(dev):
        stream = torch.cuda.current_stream(dev)
        key = ('accumulate', dev.index, stream.cuda_stream, threading.get_ident())
        with _ws_lock:
            ws = _workspaces.setdefault(key, Workspace(dev))
        ck_capacity = max(ws.ck_capacity, 16 * n_lines + 1024)
        # terms built in shared memory need no table; the call names the capacity its
        # largest terms need (CBC_ERR_CAPACITY, pairs_needed) and is run again
        table_cap = ws.capacity if (table and n_lines) else 0
        for _ in range(6):
            nbytes = lib.cbc_accumulate_lines_workspace_size(n_lines, n_terms, ck_capacity,
                                                             table_cap, elem)
            buf = ws.ensure(nbytes)
            rc = fn(work.data_ptr(), F, H, W, ln.data_ptr(), n_lines, tm.data_ptr(),
                    tm.element_size(), fr.data_ptr(), fr.element_size(), n_terms, max_val,
                    kernel, in_ov, out_ov, buf.data_ptr(), buf.numel(), ck_capacity, table_cap,
                    stream.cuda_stream)
            if rc:
                _raise_rc(rc)
            st = _native.Status()
            if lib.cbc_read_status(buf.data_ptr(), st, stream.cuda_stream):
                _raise_rc(_native.CBC_ERR_CUDA)
            ws.last_status = st
            if st.has(_native.CBC_ERR_INDEX):
                raise IndexError(f"frames range ({int(fr.min())}, {int(fr.max())}) is outside of "
                                 f"(0, {F})")
            if st.has(_native.CBC_ERR_TERM):
                raise IndexError(f"Term index {int(tm[st.bad_line])} is out of range "
                                 f"(0, {n_terms})")
            _raise_status(st, F)
            if not st.has(_native.CBC_ERR_CAPACITY):
                ws.ck_capacity = ck_capacity
                ws.capacity = table_cap
                break
            ck_capacity = max(ck_capacity, int(st.checkpoints_needed * 1.25) + 1024)
            if table:
                table_cap = max(table_cap, int(st.pairs_needed))
            if ck_capacity > 2**31 - 1:
                raise MemoryError("too many walk checkpoints for one call")
        else:
            raise RuntimeError("workspace capacity did not converge")
    if work is not out:
        out.copy_(work)
    return out


def _accumulate_lines3d_cuda(out: torch.Tensor, ln: torch.Tensor, terms, frames, max_val: float,
                             kernel: int, in_ov: int, out_ov: int) -> torch.Tensor:
    F, D, H, W = _volumes_of(out)
    dev = out.device
    n_lines = ln.shape[0]
    tm = _as_device_ints(terms, 'terms', dev)
    if tm.numel() != n_lines:
        raise ValueError(f"Term indices ({tm.numel()}) is incompatible with number of lines "
                         f"({n_lines})")
    fr = _as_device_ints(frames, 'frames', dev)
    n_terms = fr.numel()
    work = out if out.is_contiguous() else out.contiguous()
    elem = 4 if out.dtype == torch.float32 else 8
    lib = _native.lib()
    fn = lib.cbc_accumulate_lines_3d_f32 if elem == 4 else lib.cbc_accumulate_lines_3d_f64

    def check(st):
        if st.has(_native.CBC_ERR_INDEX):
            raise IndexError(f"frames range ({int(fr.min())}, {int(fr.max())}) is outside of "
                             f"(0, {F})")
        if st.has(_native.CBC_ERR_TERM):
            raise IndexError(f"Term index {int(tm[st.bad_line])} is out of range (0, {n_terms})")

    _run3(lambda buf, ck, t, stream: fn(
              work.data_ptr(), F, D, H, W, ln.data_ptr(), n_lines, tm.data_ptr(),
              tm.element_size(), fr.data_ptr(), fr.element_size(), n_terms, max_val, kernel,
              in_ov, out_ov, buf.data_ptr(), buf.numel(), ck, t, stream),
          lambda ck, t: lib.cbc_accumulate_lines_3d_workspace_size(n_lines, n_terms, ck, t, elem),
          dev, 'accumulate3d', F, n_lines, in_ov != out_ov, check,
          columns=lambda: _columns3(ln, max(D, H, W)))
    if work is not out:
        out.copy_(work)
    return out


def accumulate_lines(out, lines, terms, frames, max_val: float = 1.0,
                     kernel: str = 'rectangular', in_overlap: str = 'sum',
                     out_overlap: str = 'sum'):
    """Accumulate thick lines grouped into terms across frames (reference:
    cbclib_v2/_src/functions.py:195-233).

    Args:
        out: Output frames (..., H, W), float32 or float64, updated in place (CUDA
            arrays on their device; host arrays staged while the device is 'cuda').
        lines: (N, 5) rows [x0, y0, x1, y1, width], xy order.
        terms: (N,) term index of each line.
        frames: (T,) frame index of each term into the flattened leading dims of ``out``.
        max_val: peak value of a line's profile.
        kernel: 'biweight', 'gaussian', 'parabolic', 'rectangular' or 'triangular'.
        in_overlap: how a term combines its own lines, 'sum' or 'max'.
        out_overlap: how terms combine into ``out``, 'sum' or 'max'.

    Returns:
        ``out``.
    """
    if kernel not in _native.KERNELS:
        raise ValueError(f"kernel is missing for {kernel}")
    if in_overlap not in _native.OVERLAPS or out_overlap not in _native.OVERLAPS:
        raise ValueError(f"Invalid overlap keyword: {in_overlap}, {out_overlap}")
    k = _native.KERNELS[kernel]
    iov, oov = _native.OVERLAPS[in_overlap], _native.OVERLAPS[out_overlap]
    return _on_device(out, 'accumulate_lines',
                      lambda dev_out: _accumulate_lines_cuda(dev_out, lines, terms, frames,
                                                             max_val, k, iov, oov))
