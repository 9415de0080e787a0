"""draw_lines inside ndimage.deferred_errors(): calls queue without waiting for the
GPU and their device status is checked when the block exits.  The frames match the
checked calls, an index error raises on exit, and a call whose walks outgrew the
workspace (it drew nothing) is run again on exit."""
import numpy as np
import pytest
import torch

from cbclib_v2_gb300 import draw_lines, ndimage, workloads

pytestmark = pytest.mark.gpu


def test_deferred_calls_match_checked_calls(cuda):
    ls = workloads.detector_stack(seed=31, F=3, H=400, W=420, mean_lines=800)
    lines = torch.from_numpy(ls.lines.astype(np.float32)).cuda()
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).cuda()
    want = torch.zeros(ls.shape, device='cuda')
    got = torch.zeros(ls.shape, device='cuda')
    for k in range(3):
        draw_lines(want, lines + k, idxs, 1.0 + k, 'gaussian', 'max')
    with ndimage.deferred_errors():
        for k in range(3):
            draw_lines(got, lines + k, idxs, 1.0 + k, 'gaussian', 'max')
    assert torch.equal(got, want)


def test_deferred_index_error_raises_on_exit(cuda):
    lines = torch.tensor([[2.0, 2, 30, 20, 2.0], [5, 30, 40, 3, 1.5]], device='cuda')
    out = torch.zeros((2, 40, 50), device='cuda')
    good = torch.tensor([0, 1], dtype=torch.int32, device='cuda')
    bad = torch.tensor([0, 2], dtype=torch.int32, device='cuda')
    with pytest.raises(IndexError):
        with ndimage.deferred_errors():
            draw_lines(out, lines, good, 1.0, 'rectangular', 'max')
            draw_lines(out, lines * 0.5, bad, 1.0, 'rectangular', 'sum')
    ref = torch.zeros((2, 40, 50), device='cuda')
    draw_lines(ref, lines, good, 1.0, 'rectangular', 'max')
    assert torch.equal(out, ref)             # the first call drew, the bad one did not


def test_deferred_capacity_overflow_runs_again(cuda):
    ndimage.release_scratch()                 # a fresh workspace, sized by the first call
    short = torch.tensor([[3.0, 3, 9, 5, 1.0]], device='cuda')
    W = 30000
    y = torch.tensor([2.5, 4.5, 6.5], device='cuda')
    long = torch.stack([torch.full((3,), 10.0, device='cuda'), y,
                        torch.full((3,), W - 10.0, device='cuda'), y,
                        torch.full((3,), 1.5, device='cuda')], 1)
    got = torch.zeros((1, 10, W), device='cuda')
    want = torch.zeros((1, 10, W), device='cuda')
    for out in (want,):
        draw_lines(out, short, None, 1.0, 'biweight', 'max')
        draw_lines(out, long, None, 1.0, 'biweight', 'max')
    ndimage.release_scratch()
    with ndimage.deferred_errors():
        draw_lines(got, short, None, 1.0, 'biweight', 'max')
        draw_lines(got, long, None, 1.0, 'biweight', 'max')   # ~11,000 walk checkpoints
    assert torch.equal(got, want) and bool((got > 0).sum() > 1000)
