"""The no-allocation entry point (cbc_draw_lines_f32_noalloc) against the workspace
entry point, called through the C ABI.

It exists for callers that cannot give the library device memory: an acquisition
loop that reserves its whole device budget before a run and must not stall on
cudaMalloc or run out of memory half-way, or a plugin whose host framework owns all
device memory.  Its scratch is a fixed array inside the library, so it has limits
(CBC_NOALLOC_MAX_LINES lines, CBC_NOALLOC_MAX_CHECKPOINTS walk checkpoints).  Two
calls in a row must each match the workspace entry point, which also shows that the
second call does not see what the first left in the shared array.  This file is
collected last so a failure here leaves every other test already run.
"""
import numpy as np
import pytest
import torch

from cbclib_v2_gb300 import _native, draw_lines, workloads

pytestmark = pytest.mark.gpu

SUM_RTOL = 1e-5
SUM_ATOL = 1e-7


def _noalloc(out, lines, idxs, max_val, kernel, overlap):
    lib = _native.lib()
    F = int(np.prod(out.shape[:-2]))
    H, W = out.shape[-2:]
    return lib.cbc_draw_lines_f32_noalloc(
        out.data_ptr(), F, H, W, lines.data_ptr(), lines.shape[0],
        None if idxs is None else idxs.data_ptr(), 0 if idxs is None else idxs.element_size(),
        max_val, _native.KERNELS[kernel], _native.OVERLAPS[overlap],
        torch.cuda.current_stream().cuda_stream)


def _noalloc_raw(out, lines, n_frames):
    return _native.lib().cbc_draw_lines_f32_noalloc(
        out.data_ptr(), n_frames, 1, 1, lines.data_ptr(), lines.shape[0], None, 0, 1.0, 0, 0,
        torch.cuda.current_stream().cuda_stream)


def _workspace_result(out0, lines, idxs, max_val, kernel, overlap):
    out = out0.clone()
    draw_lines(out, lines, idxs, max_val, kernel, overlap)
    return out


def test_noalloc_matches_workspace_entry_point():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ls = workloads.detector_stack(seed=11, F=3, H=500, W=610, mean_lines=900)
    lines = torch.from_numpy(ls.lines.astype(np.float32)).cuda()
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).cuda()
    assert lines.shape[0] <= _native.NOALLOC_MAX_LINES
    # first call: sum into a non-zero frame stack; second call: max into zeros
    calls = [(torch.full(ls.shape, 0.25, device='cuda'), 2.0, 'biweight', 'sum'),
             (torch.zeros(ls.shape, device='cuda'), 1.0, 'gaussian', 'max')]
    for out0, max_val, kernel, overlap in calls:
        want = _workspace_result(out0, lines, idxs, max_val, kernel, overlap).cpu().numpy()
        got = out0.clone()
        rc = _noalloc(got, lines, idxs, max_val, kernel, overlap)
        assert rc == _native.CBC_OK, _native.last_error()
        got = got.cpu().numpy()
        assert (got != out0.cpu().numpy()).any()
        if overlap == 'max':
            assert np.array_equal(got, want)
        else:
            tol = SUM_RTOL * np.abs(want) + SUM_ATOL * max_val
            assert np.all(np.abs(got.astype(np.float64) - want) <= tol)


def test_noalloc_limits_and_errors():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    single = torch.zeros((40, 50), device='cuda')
    too_many = torch.zeros((_native.NOALLOC_MAX_LINES + 1, 5), device='cuda')
    rc = _noalloc(single, too_many, None, 1.0, 'rectangular', 'sum')
    assert rc == _native.CBC_ERR_INVALID and 'maximum' in _native.last_error()
    out = torch.zeros((2, 40, 50), device='cuda')
    lines = torch.tensor([[2, 2, 30, 20, 2.0], [5, 30, 40, 3, 1.5]], device='cuda')
    rc = _noalloc(out, lines, torch.tensor([0, 2], dtype=torch.int32, device='cuda'), 1.0,
                  'rectangular', 'max')
    assert rc == _native.CBC_ERR_INDEX and '(0, 2)' in _native.last_error()
    assert float(out.abs().sum()) == 0.0
    # frame counts beyond 32 bits are rejected on the host
    rc = _noalloc_raw(out, lines, 1 << 31)
    assert rc == _native.CBC_ERR_INVALID and 'n_frames' in _native.last_error()


def test_noalloc_index_widths_and_frame_per_line():
    """int64 frame indices, and no indices with one frame per line (line i into frame
    i), against the workspace entry point and the oracle"""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import oracle
    ls = workloads.detector_stack(seed=12, F=4, H=300, W=350, mean_lines=500)
    lines32 = ls.lines.astype(np.float32)
    lines = torch.from_numpy(lines32).cuda()
    for idxs in (torch.from_numpy(ls.idxs.astype(np.int64)).cuda(), None):
        shape = ls.shape if idxs is not None else (lines.shape[0], 40, 60)
        ix = ls.idxs if idxs is not None else None
        for kernel, overlap in (('gaussian', 'max'), ('triangular', 'sum')):
            want = _workspace_result(torch.zeros(shape, device='cuda'), lines, idxs, 1.5, kernel,
                                     overlap).cpu().numpy()
            ref = oracle.draw_lines(np.zeros(shape, np.float32), lines32, ix, 1.5, kernel,
                                    overlap, 4)
            got = torch.zeros(shape, device='cuda')
            rc = _noalloc(got, lines, idxs, 1.5, kernel, overlap)
            assert rc == _native.CBC_OK, _native.last_error()
            got = got.cpu().numpy()
            assert got.any()
            if overlap == 'max':
                assert np.array_equal(got, want) and np.array_equal(got, ref)
            else:
                for other in (want, ref):
                    tol = SUM_RTOL * np.abs(other) + SUM_ATOL * 1.5
                    assert np.all(np.abs(got.astype(np.float64) - other) <= tol)


def test_noalloc_checkpoint_limit_draws_nothing():
    """walks needing more than CBC_NOALLOC_MAX_CHECKPOINTS checkpoints (one per 16
    columns): CBC_ERR_CAPACITY and the frames untouched; the next call is clean"""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    W = 200000
    n = 25                                   # 25 walks of ~12,500 checkpoints each
    y = np.linspace(1.5, 6.5, n)
    lines = torch.tensor(np.c_[np.full(n, 10.0), y, np.full(n, W - 10.0), y, np.ones(n)],
                         dtype=torch.float32, device='cuda')
    assert n * (W - 20) // 16 > _native.NOALLOC_MAX_CHECKPOINTS
    out = torch.full((1, 8, W), 0.5, device='cuda')
    rc = _noalloc(out, lines, None, 1.0, 'rectangular', 'sum')
    assert rc == _native.CBC_ERR_CAPACITY and 'checkpoints' in _native.last_error()
    assert bool(torch.all(out == 0.5))
    few = lines[:3].contiguous()
    got = torch.full((1, 8, W), 0.5, device='cuda')
    assert _noalloc(got, few, None, 1.0, 'rectangular', 'max') == _native.CBC_OK
    want = _workspace_result(torch.full((1, 8, W), 0.5, device='cuda'), few, None, 1.0,
                             'rectangular', 'max')
    assert torch.equal(got, want) and bool((got == 1.0).any())
