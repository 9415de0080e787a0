"""draw_lines on page-locked host frames: the kernels draw into a device scratch at
the overlap's identity and combine the drawn pixels into the host frames through
their device mapping (no frame copies).  The result is the device path's, index
errors leave the frames untouched, and the scratch is back at the identity after
every call (overlap and dtype changes refill it)."""
import numpy as np
import pytest
import torch

from cbclib_v2_gb300 import draw_lines, ndimage

pytestmark = pytest.mark.gpu


def random_lines(rng, n, H, W):
    lines = np.empty((n, 5))
    lines[:, 0] = rng.uniform(-5, W + 5, n)
    lines[:, 1] = rng.uniform(-5, H + 5, n)
    lines[:, 2] = lines[:, 0] + rng.uniform(-25, 25, n)
    lines[:, 3] = lines[:, 1] + rng.uniform(-25, 25, n)
    lines[:, 4] = rng.uniform(0.5, 4, n)
    return lines


def device_result(base, lines, idxs, kernel, overlap, max_val=1.7):
    ref = base.cuda()
    draw_lines(ref, torch.tensor(lines, dtype=base.dtype, device='cuda'),
               None if idxs is None else torch.tensor(idxs, device='cuda'), max_val, kernel,
               overlap)
    return ref.cpu()


def same(got, want, overlap):
    if overlap == 'max':
        assert torch.equal(got, want)
    else:                                  # the sum is formed in another order
        torch.testing.assert_close(got, want, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("overlap", ['sum', 'max'])
def test_host_frames_match_device_path(cuda, dtype, overlap):
    rng = np.random.default_rng(21)
    F, H, W = 11, 48, 70
    lines = random_lines(rng, 300, H, W)
    idxs = rng.integers(0, F, 300)
    base = torch.rand((F, H, W), dtype=dtype) - 0.3       # negative pixels too
    host = base.clone().pin_memory()
    assert host.is_pinned()
    out = draw_lines(host, torch.tensor(lines, dtype=dtype), torch.tensor(idxs), 1.7, 'gaussian',
                     overlap)
    assert out is host
    same(host, device_result(base, lines, idxs, 'gaussian', overlap), overlap)


def test_scratch_identity_kept_across_calls(cuda):
    """max, then sum, then max again on the same frames; each call's result is the
    device path's, so the scratch held the right identity every time"""
    rng = np.random.default_rng(22)
    F, H, W = 5, 40, 44
    base = torch.rand((F, H, W))
    host = base.clone().pin_memory()
    ref = base.cuda()
    for k, (kernel, overlap) in enumerate([('biweight', 'max'), ('triangular', 'sum'),
                                           ('biweight', 'max'), ('parabolic', 'max'),
                                           ('triangular', 'sum')]):
        lines = random_lines(rng, 60, H, W)
        idxs = rng.integers(0, F, 60)
        draw_lines(host, lines, idxs, 1.0 + k, kernel, overlap)
        draw_lines(ref, torch.tensor(lines, dtype=torch.float32, device='cuda'),
                   torch.tensor(idxs, device='cuda'), 1.0 + k, kernel, overlap)
        same(host, ref.cpu(), overlap)
        host.copy_(ref.cpu())             # carry on from the same frames


def test_scratch_identity_after_smaller_stacks(cuda):
    """a large max stack, a small sum stack (which fills only its own part of the
    cached scratch), then a middle-sized sum stack: the last call must fill the part
    the small call left at the max identity"""
    rng = np.random.default_rng(28)
    for (F, H, W), overlap in (((6, 50, 60), 'max'), ((2, 30, 30), 'sum'),
                               ((5, 44, 50), 'sum')):
        lines = random_lines(rng, 80, H, W)
        idxs = rng.integers(0, F, 80)
        base = torch.rand((F, H, W))
        host = base.clone().pin_memory()
        draw_lines(host, lines, idxs, 1.2, 'parabolic', overlap)
        same(host, device_result(base, lines, idxs, 'parabolic', overlap, 1.2), overlap)


def test_host_frames_one_line_per_frame(cuda):
    rng = np.random.default_rng(23)
    F, H, W = 6, 40, 40
    lines = random_lines(rng, F, H, W)
    host = torch.zeros((F, H, W)).pin_memory()
    draw_lines(host, lines, None, 1.7, 'biweight', 'max')
    assert torch.equal(host, device_result(torch.zeros((F, H, W)), lines, None, 'biweight', 'max'))


def test_host_frames_index_error_leaves_frames(cuda):
    rng = np.random.default_rng(24)
    F, H, W = 5, 32, 32
    lines = random_lines(rng, 20, H, W)
    idxs = rng.integers(0, F, 20)
    idxs[7] = F
    base = torch.rand((F, H, W))
    host = base.clone().pin_memory()
    with pytest.raises(IndexError):
        draw_lines(host, lines, idxs, 1.0, 'biweight', 'sum')
    assert torch.equal(host, base)
    idxs[7] = 0                            # and the next call is clean
    draw_lines(host, lines, idxs, 1.0, 'biweight', 'sum')
    same(host, device_result(base, lines, idxs, 'biweight', 'sum', 1.0), 'sum')


def test_pageable_frames(cuda):
    """NumPy arrays and unpinned tensors: drawn in place through the pageable mapping
    where the device reads and writes pageable memory coherently (NVLink-C2C), copied
    up and down otherwise; the result is the device path's either way"""
    rng = np.random.default_rng(25)
    F, H, W = 4, 30, 30
    lines = random_lines(rng, 12, H, W)
    lines[3, 0] = 3e6                   # far away, a legal line
    idxs = rng.integers(0, F, 12)
    for host in (torch.zeros((F, H, W), dtype=torch.float64),
                 np.zeros((F, H, W), dtype=np.float64)):
        draw_lines(host, lines, idxs, 1.0, 'parabolic', 'max')
        want = device_result(torch.zeros((F, H, W), dtype=torch.float64), lines, idxs,
                             'parabolic', 'max', 1.0)
        assert torch.equal(torch.as_tensor(host), want)


@pytest.mark.parametrize("overlap", ['sum', 'max'])
def test_numpy_frames_in_place(cuda, overlap):
    """a NumPy stack updated in place (the array object and its memory are kept), with
    negative pixels, float32 and float64, against the device path"""
    from cbclib_v2_gb300 import _native
    rng = np.random.default_rng(26)
    F, H, W = 7, 52, 61
    lines = random_lines(rng, 200, H, W)
    idxs = rng.integers(0, F, 200).astype(np.int32)
    for dtype in (np.float32, np.float64):
        base = (rng.random((F, H, W)) - 0.2).astype(dtype)
        host = base.copy()
        ptr = host.ctypes.data
        out = draw_lines(host, lines.astype(dtype), idxs, 1.3, 'triangular', overlap)
        assert out is host and host.ctypes.data == ptr
        want = device_result(torch.from_numpy(base), lines, idxs, 'triangular', overlap, 1.3)
        same(torch.from_numpy(host), want, overlap)
    mode = _native.host_access(host.ctypes.data)
    assert mode in (_native.HOST_PAGEABLE, _native.HOST_NONE)


def test_numpy_lines_and_indices_read_in_place(cuda):
    """NumPy frames, lines and int32/int64 indices (read by the kernels where they lie
    on devices that reach pageable memory), float32 and float64, against the device
    path; a float64 line array with float32 frames is converted first"""
    rng = np.random.default_rng(27)
    F, H, W = 5, 47, 66
    lines = random_lines(rng, 150, H, W)
    for dtype, idx_dtype in ((np.float32, np.int32), (np.float64, np.int64), (np.float32, np.int64)):
        idxs = rng.integers(0, F, 150).astype(idx_dtype)
        base = rng.random((F, H, W)).astype(dtype)
        host = base.copy()
        ln = np.ascontiguousarray(lines.astype(dtype))
        draw_lines(host, ln, idxs, 1.1, 'biweight', 'max')
        want = device_result(torch.from_numpy(base), lines, idxs, 'biweight', 'max', 1.1)
        same(torch.from_numpy(host), want, 'max')
    host = np.zeros((F, H, W), np.float32)
    draw_lines(host, lines, rng.integers(0, F, 150), 1.1, 'biweight', 'max')   # float64 lines
    assert host.any()
