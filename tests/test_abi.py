"""The C-ABI library builds, loads and exports every symbol that include/*.h declares;
host-side argument validation works without a GPU (no kernel is launched)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from cbclib_v2_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, 'include', '*.h')):
        text = open(h).read()
        names.update(re.findall(r'CBC_API\s+[\w\s\*]*?\b(cbc_\w+)\s*\(', text))
    return names


def test_exports_every_declared_symbol():
    lib = _native.lib()
    names = declared_symbols()
    assert {'cbc_draw_lines_f32', 'cbc_draw_lines_f64', 'cbc_read_status'} <= names
    for n in names:
        assert hasattr(lib, n), n
    assert set(_native.EXPORTS) <= names


def test_noalloc_limits_match_the_header():
    text = open(os.path.join(ROOT, 'include', 'cbc_draw_lines.h')).read()
    defs = dict(re.findall(r'#define\s+(CBC_NOALLOC_MAX_\w+)\s+(\d+)', text))
    assert int(defs['CBC_NOALLOC_MAX_LINES']) == _native.NOALLOC_MAX_LINES
    assert int(defs['CBC_NOALLOC_MAX_CHECKPOINTS']) == _native.NOALLOC_MAX_CHECKPOINTS


def test_noalloc_rejects_frame_counts_beyond_32_bits():
    """rejected on the host, before any device call"""
    lib = _native.lib()
    rc = lib.cbc_draw_lines_f32_noalloc(None, 1 << 31, 1, 1, None, 1, None, 0, 1.0, 0, 0, None)
    assert rc == _native.CBC_ERR_INVALID and 'n_frames' in _native.last_error()


def test_version():
    assert b'sm_103a' in _native.lib().cbc_version()


def test_workspace_size():
    lib = _native.lib()
    a = lib.cbc_draw_lines_workspace_size(64, 2167, 2070, 128000, 400000, 900000, 4, None)
    b = lib.cbc_draw_lines_workspace_size(64, 2167, 2070, 128000, 800000, 900000, 4, None)
    c = lib.cbc_draw_lines_workspace_size(64, 2167, 2070, 128000, 400000, 900000, 8, None)
    d = lib.cbc_draw_lines_workspace_size(64, 2167, 2070, 128000, 400000, 1800000, 4, None)
    assert 0 < a < b and a < c and a < d
    assert b - a >= 4 * 400000 and d - a >= 16 * 900000
    t = _native.Tuning(7, 64, 16, 0)   # tile_w not a multiple of 4
    assert lib.cbc_draw_lines_workspace_size(1, 64, 64, 10, 100, 100, 4, ctypes.pointer(t)) == 0


@pytest.mark.parametrize("args,msg", [
    (dict(kernel=9), 'kernel'),
    (dict(overlap=3), 'overlap'),
    (dict(n_frames=3), 'incompatible'),
    (dict(idx_bytes=2, idxs=1), 'idx_bytes'),
    (dict(n_lines=-1), 'negative'),
])
def test_host_validation(args, msg):
    lib = _native.lib()
    p = dict(out=None, n_frames=1, H=10, W=10, lines=None, n_lines=5, idxs=None, idx_bytes=0,
             max_val=1.0, kernel=0, overlap=0, ws=None, ws_bytes=0, cap=0)
    p.update(args)
    rc = lib.cbc_draw_lines_f32(p['out'], p['n_frames'], p['H'], p['W'], p['lines'],
                                p['n_lines'], p['idxs'], p['idx_bytes'], p['max_val'],
                                p['kernel'], p['overlap'], p['ws'], p['ws_bytes'], p['cap'],
                                p['cap'], None, None)
    assert rc == _native.CBC_ERR_INVALID
    assert msg in _native.last_error()


def test_workspace_too_small_is_rejected():
    lib = _native.lib()
    rc = lib.cbc_draw_lines_f32(None, 1, 10, 10, None, 0, None, 0, 1.0, 0, 0, None, 16, 100,
                                100, None, None)
    assert rc == _native.CBC_ERR_INVALID and 'workspace' in _native.last_error()
