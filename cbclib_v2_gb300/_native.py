"""ctypes binding of the C ABI in include/cbc_draw_lines.h (libcbc_gb300.so).

The library is the only compute path of this package: when it cannot be loaded the
package raises instead of falling back to anything else.
"""
import ctypes
import os
import threading

from . import build as _build

CBC_OK, CBC_ERR_INVALID, CBC_ERR_INDEX, CBC_ERR_CAPACITY, CBC_ERR_CUDA, CBC_ERR_RANGE = range(6)
CBC_ERR_TERM = 6
MAX_WALK = 1 << 22

STRATEGY_AUTO, STRATEGY_TILES, STRATEGY_LINES = 0, 1, 2

KERNELS = {'biweight': 0, 'gaussian': 1, 'parabolic': 2, 'rectangular': 3, 'triangular': 4}
OVERLAPS = {'sum': 0, 'max': 1}


class Tuning(ctypes.Structure):
    """cbc_tuning: render tile shape and lines per shared-memory chunk (0 = default)."""
    _fields_ = [('tile_w', ctypes.c_int32), ('tile_h', ctypes.c_int32),
                ('chunk_lines', ctypes.c_int32), ('threads', ctypes.c_int32),
                ('strategy', ctypes.c_int32), ('reserved', ctypes.c_int32)]


class Status(ctypes.Structure):
    """cbc_status: device-side result flags of the last call on a workspace."""
    _fields_ = [('flags', ctypes.c_int32), ('strategy', ctypes.c_int32),
                ('bad_line', ctypes.c_int64), ('idx_min', ctypes.c_int64),
                ('idx_max', ctypes.c_int64), ('pairs_needed', ctypes.c_int64),
                ('checkpoints_needed', ctypes.c_int64)]

    def has(self, code: int) -> bool:
        return bool(self.flags & (1 << code))


class Profile(ctypes.Structure):
    """cbc_profile: accumulated per-stage device milliseconds of profiled calls."""
    _fields_ = [('calls', ctypes.c_int32), ('launches', ctypes.c_int32),
                ('ms_prep', ctypes.c_double), ('ms_offsets', ctypes.c_double),
                ('ms_fill', ctypes.c_double), ('ms_render', ctypes.c_double)]


_lock = threading.Lock()
_lib = None

# every symbol declared in include/cbc_draw_lines.h
EXPORTS = ('cbc_draw_lines_workspace_size', 'cbc_draw_lines_f32', 'cbc_draw_lines_f64',
           'cbc_draw_lines_csr_f32', 'cbc_draw_lines_csr_f64',
           'cbc_draw_lines_f32_noalloc', 'cbc_draw_lines_backward_workspace_size',
           'cbc_draw_lines_backward_f32', 'cbc_draw_lines_backward_f64', 'cbc_read_status',
           'cbc_profile_enable', 'cbc_profile_read', 'cbc_last_error', 'cbc_version',
           'cbc_accumulate_lines_workspace_size', 'cbc_accumulate_lines_f32',
           'cbc_accumulate_lines_f64', 'cbc_draw_lines_3d_workspace_size',
           'cbc_draw_lines_3d_f32', 'cbc_draw_lines_3d_f64',
           'cbc_accumulate_lines_3d_workspace_size', 'cbc_accumulate_lines_3d_f32',
           'cbc_accumulate_lines_3d_f64', 'cbc_squared_loss_backward_f32',
           'cbc_squared_loss_backward_f64', 'cbc_draw_lines_max_winner_f32',
           'cbc_draw_lines_backward_ex_f32', 'cbc_draw_lines_backward_ex_f64',
           'cbc_squared_loss_step_workspace_size', 'cbc_squared_loss_step_f32',
           'cbc_squared_loss_step_sum_f32',
           'cbc_status_bytes', 'cbc_copy_status_async', 'cbc_decode_status',
           'cbc_adam_step_f32', 'cbc_draw_lines_host_f32', 'cbc_draw_lines_host_f64',
           'cbc_host_access', 'cbc_draw_lines_3d_backward_workspace_size',
           'cbc_draw_lines_3d_backward_f32', 'cbc_draw_lines_3d_backward_f64')

HOST_NONE, HOST_MAPPED, HOST_PAGEABLE = 0, 1, 2

NO_WINNER = 0x7f7f7f7f

NOALLOC_MAX_LINES = 16384
NOALLOC_MAX_CHECKPOINTS = 262144


def _declare(lib):
    p, i64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32
    lib.cbc_draw_lines_workspace_size.argtypes = [i64, i64, i64, i64, i64, i64, i32,
                                                  ctypes.POINTER(Tuning)]
    lib.cbc_draw_lines_workspace_size.restype = ctypes.c_size_t
    for sfx, real in (('f32', ctypes.c_float), ('f64', ctypes.c_double)):
        f = getattr(lib, 'cbc_draw_lines_' + sfx)
        f.argtypes = [p, i64, i64, i64, p, i64, p, i32, real, i32, i32, p, ctypes.c_size_t,
                      i64, i64, ctypes.POINTER(Tuning), p]
        f.restype = ctypes.c_int
    for sfx, real in (('f32', ctypes.c_float), ('f64', ctypes.c_double)):
        f = getattr(lib, 'cbc_draw_lines_csr_' + sfx)
        f.argtypes = [p, i64, i64, i64, p, i64, p, real, i32, i32, p, ctypes.c_size_t, i64, i64,
                      ctypes.POINTER(Tuning), p]
        f.restype = ctypes.c_int
    lib.cbc_draw_lines_f32_noalloc.argtypes = [p, i64, i64, i64, p, i64, p, i32, ctypes.c_float,
                                               i32, i32, p]
    lib.cbc_draw_lines_f32_noalloc.restype = ctypes.c_int
    lib.cbc_draw_lines_backward_workspace_size.argtypes = [i64, i64, i32]
    lib.cbc_draw_lines_backward_workspace_size.restype = ctypes.c_size_t
    for sfx, real in (('f32', ctypes.c_float), ('f64', ctypes.c_double)):
        f = getattr(lib, 'cbc_draw_lines_backward_' + sfx)
        f.argtypes = [p, i64, i64, i64, p, i64, p, i32, real, i32, i32, p, p, p, p, p,
                      ctypes.c_size_t, i64, p]
        f.restype = ctypes.c_int
    lib.cbc_accumulate_lines_workspace_size.argtypes = [i64, i64, i64, i64, i32]
    lib.cbc_accumulate_lines_workspace_size.restype = ctypes.c_size_t
    for sfx, real in (('f32', ctypes.c_float), ('f64', ctypes.c_double)):
        f = getattr(lib, 'cbc_accumulate_lines_' + sfx)
        f.argtypes = [p, i64, i64, i64, p, i64, p, i32, p, i32, i64, real, i32, i32, i32, p,
                      ctypes.c_size_t, i64, i64, p]
        f.restype = ctypes.c_int
    lib.cbc_draw_lines_3d_workspace_size.argtypes = [i64, i64, i32]
    lib.cbc_draw_lines_3d_workspace_size.restype = ctypes.c_size_t
    lib.cbc_accumulate_lines_3d_workspace_size.argtypes = [i64, i64, i64, i64, i32]
    lib.cbc_accumulate_lines_3d_workspace_size.restype = ctypes.c_size_t
    for sfx, real in (('f32', ctypes.c_float), ('f64', ctypes.c_double)):
        f = getattr(lib, 'cbc_draw_lines_3d_' + sfx)
        f.argtypes = [p, i64, i64, i64, i64, p, i64, p, i32, real, i32, i32, p, ctypes.c_size_t,
                      i64, p]
        f.restype = ctypes.c_int
        f = getattr(lib, 'cbc_accumulate_lines_3d_' + sfx)
        f.argtypes = [p, i64, i64, i64, i64, p, i64, p, i32, p, i32, i64, real, i32, i32, i32, p,
                      ctypes.c_size_t, i64, i64, p]
        f.restype = ctypes.c_int
    for sfx, real in (('f32', ctypes.c_float), ('f64', ctypes.c_double)):
        f = getattr(lib, 'cbc_squared_loss_backward_' + sfx)
        f.argtypes = [p, p, i64, i64, i64, p, i64, p, i32, real, i32, i32, p, p, p, p,
                      ctypes.c_size_t, i64, p]
        f.restype = ctypes.c_int
    lib.cbc_draw_lines_max_winner_f32.argtypes = [p, p, p, i64, i64, i64, p, i64, p, i32,
                                                  ctypes.c_float, i32, p, ctypes.c_size_t,
                                                  i64, i64, p]
    lib.cbc_draw_lines_max_winner_f32.restype = ctypes.c_int
    for sfx, real in (('f32', ctypes.c_float), ('f64', ctypes.c_double)):
        f = getattr(lib, 'cbc_draw_lines_backward_ex_' + sfx)
        f.argtypes = [p, p, i64, i64, i64, p, i64, p, i32, real, i32, i32, p, p, p, i32, p, p,
                      p, ctypes.c_size_t, i64, p]
        f.restype = ctypes.c_int
    lib.cbc_squared_loss_step_workspace_size.argtypes = [i64, i64, i64, i64, i64, i64]
    lib.cbc_squared_loss_step_workspace_size.restype = ctypes.c_size_t
    lib.cbc_squared_loss_step_f32.argtypes = [p, i64, i64, i64, p, i64, p, i32, ctypes.c_float,
                                              i32, p, p, p, p, ctypes.c_size_t, i64, i64, p]
    lib.cbc_squared_loss_step_f32.restype = ctypes.c_int
    lib.cbc_squared_loss_step_sum_f32.argtypes = [p, p, i64, i64, i64, p, i64, p, i32,
                                                  ctypes.c_float, i32, p, p, p, ctypes.c_size_t,
                                                  i64, i64, p]
    lib.cbc_squared_loss_step_sum_f32.restype = ctypes.c_int
    for sfx, real in (('f32', ctypes.c_float), ('f64', ctypes.c_double)):
        f = getattr(lib, 'cbc_draw_lines_host_' + sfx)
        f.argtypes = [p, i64, i64, i64, p, i64, p, i32, real, i32, i32, p, i32, p,
                      ctypes.c_size_t, i64, i64, p, p]
        f.restype = ctypes.c_int
    lib.cbc_adam_step_f32.argtypes = [p, p, p, p, i64, i64, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_float, ctypes.c_float, ctypes.c_float, p]
    lib.cbc_adam_step_f32.restype = ctypes.c_int
    lib.cbc_status_bytes.argtypes = []
    lib.cbc_status_bytes.restype = ctypes.c_size_t
    lib.cbc_copy_status_async.argtypes = [p, p, p]
    lib.cbc_copy_status_async.restype = ctypes.c_int
    lib.cbc_decode_status.argtypes = [p, ctypes.POINTER(Status)]
    lib.cbc_decode_status.restype = ctypes.c_int
    lib.cbc_read_status.argtypes = [p, ctypes.POINTER(Status), p]
    lib.cbc_read_status.restype = ctypes.c_int
    lib.cbc_profile_enable.argtypes = [i32]
    lib.cbc_profile_enable.restype = ctypes.c_int
    lib.cbc_profile_read.argtypes = [ctypes.POINTER(Profile), i32]
    lib.cbc_profile_read.restype = ctypes.c_int
    lib.cbc_last_error.argtypes = []
    lib.cbc_last_error.restype = ctypes.c_char_p
    lib.cbc_version.argtypes = []
    lib.cbc_version.restype = ctypes.c_char_p
    lib.cbc_host_access.argtypes = [p, ctypes.POINTER(i32)]
    lib.cbc_host_access.restype = ctypes.c_int
    lib.cbc_draw_lines_3d_backward_workspace_size.argtypes = [i64, i64, i32]
    lib.cbc_draw_lines_3d_backward_workspace_size.restype = ctypes.c_size_t
    for sfx, real in (('f32', ctypes.c_float), ('f64', ctypes.c_double)):
        f = getattr(lib, 'cbc_draw_lines_3d_backward_' + sfx)
        f.argtypes = [p, i64, i64, i64, i64, p, i64, p, i32, real, i32, i32, p, p, p, p, p,
                      ctypes.c_size_t, i64, p]
        f.restype = ctypes.c_int


def library_path() -> str:
    return _build.LIB


def lib():
    """Load (building first if the sources are newer) and return the native library."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                path = _build.build()
                if not os.path.exists(path):
                    raise RuntimeError(f"native library {path} is missing")
                handle = ctypes.CDLL(path)
                _declare(handle)
                _lib = handle
    return _lib


def last_error() -> str:
    msg = lib().cbc_last_error()
    return msg.decode() if msg else ''


def host_access(ptr: int) -> int:
    """HOST_MAPPED, HOST_PAGEABLE or HOST_NONE: how the current device reaches the host
    memory at ``ptr`` (cbc_host_access)"""
    mode = ctypes.c_int32(HOST_NONE)
    rc = lib().cbc_host_access(ctypes.c_void_p(ptr), ctypes.byref(mode))
    if rc:
        raise RuntimeError(f"cbc_host_access failed: {last_error()}")
    return int(mode.value)


def profile_enable(on: bool) -> bool:
    """Switch the per-stage CUDA-event timing of the library on or off."""
    return bool(lib().cbc_profile_enable(1 if on else 0))


def profile_read(reset: bool = True) -> Profile:
    """Accumulated per-stage device times of the profiled calls (waits for them)."""
    p = Profile()
    rc = lib().cbc_profile_read(p, 1 if reset else 0)
    if rc:
        raise RuntimeError(f"cbc_profile_read failed: {last_error()}")
    return p
