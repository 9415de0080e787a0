"""draw_lines on page-locked host frames: the pipelined staging path (frame chunks
copied up, drawn and copied back on three streams) gives the device path's result,
reports index errors before any frame moves, and redraws a chunk whose walk
checkpoints did not fit."""
import numpy as np
import pytest
import torch

from cbclib_v2_gb300 import draw_lines, ndimage

pytestmark = pytest.mark.gpu


def random_lines(rng, n, H, W, long=False):
    lines = np.empty((n, 5))
    lines[:, 0] = rng.uniform(-5, W + 5, n)
    lines[:, 1] = rng.uniform(-5, H + 5, n)
    span = 3 * max(H, W) if long else 25
    lines[:, 2] = lines[:, 0] + rng.uniform(-span, span, n)
    lines[:, 3] = lines[:, 1] + rng.uniform(-span, span, n)
    lines[:, 4] = rng.uniform(0.5, 4, n)
    return lines


def device_result(base, lines, idxs, kernel, overlap, max_val=1.7):
    ref = base.cuda()
    draw_lines(ref, torch.tensor(lines, dtype=base.dtype, device='cuda'),
               None if idxs is None else torch.tensor(idxs, device='cuda'), max_val, kernel,
               overlap)
    return ref.cpu()


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("overlap", ['sum', 'max'])
def test_staged_matches_device_path(cuda, dtype, overlap):
    rng = np.random.default_rng(21)
    F, H, W = 11, 48, 70
    lines = random_lines(rng, 300, H, W)
    idxs = rng.integers(0, F, 300)
    base = torch.rand((F, H, W), dtype=dtype) * 0.5
    host = base.clone().pin_memory()
    assert host.is_pinned()
    draw_lines(host, torch.tensor(lines, dtype=dtype), torch.tensor(idxs), 1.7, 'gaussian',
               overlap)
    want = device_result(base, lines, idxs, 'gaussian', overlap)
    if overlap == 'max':
        assert torch.equal(host, want)
    else:                                  # addition order differs between two renders
        torch.testing.assert_close(host, want, rtol=1e-5, atol=1e-6)


def test_staged_one_line_per_frame(cuda):
    rng = np.random.default_rng(22)
    F, H, W = 6, 40, 40
    lines = random_lines(rng, F, H, W)
    host = torch.zeros((F, H, W)).pin_memory()
    draw_lines(host, lines, None, 1.7, 'biweight', 'max')
    assert torch.equal(host, device_result(torch.zeros((F, H, W)), lines, None, 'biweight', 'max'))


def test_staged_index_error_leaves_frames(cuda):
    rng = np.random.default_rng(23)
    F, H, W = 5, 32, 32
    lines = random_lines(rng, 20, H, W)
    idxs = rng.integers(0, F, 20)
    idxs[7] = F
    base = torch.rand((F, H, W))
    host = base.clone().pin_memory()
    with pytest.raises(IndexError):
        draw_lines(host, lines, idxs, 1.0, 'biweight', 'sum')
    assert torch.equal(host, base)


def test_staged_checkpoint_overflow_redraws_chunk(cuda):
    """with no walk checkpoints reserved per line the chunks of long lines overflow,
    draw nothing, and are drawn again synchronously"""
    rng = np.random.default_rng(24)
    F, H, W = 8, 400, 500
    lines = random_lines(rng, 800, H, W, long=True)
    idxs = rng.integers(0, F, 800)
    base = torch.zeros((F, H, W))
    host = base.clone().pin_memory()
    st = ndimage._stager(torch.device('cuda', torch.cuda.current_device()))
    st.ck_per_line = 0.0
    draw_lines(host, lines, idxs, 1.0, 'triangular', 'max')
    assert torch.equal(host, device_result(base, lines, idxs, 'triangular', 'max', 1.0))
    assert st.ck_per_line > 1.0
    again = base.clone().pin_memory()      # the learned reservation fits: no redraw
    draw_lines(again, lines, idxs, 1.0, 'triangular', 'max')
    assert torch.equal(again, host)


def test_staged_far_coordinates_take_synchronous_path(cuda):
    rng = np.random.default_rng(25)
    F, H, W = 4, 30, 30
    lines = random_lines(rng, 12, H, W)
    lines[3, 0] = 3e6                   # beyond the staging bound, a legal line
    idxs = rng.integers(0, F, 12)
    host = torch.zeros((F, H, W), dtype=torch.float64).pin_memory()
    draw_lines(host, lines, idxs, 1.0, 'parabolic', 'max')
    want = device_result(torch.zeros((F, H, W), dtype=torch.float64), lines, idxs, 'parabolic',
                         'max', 1.0)
    assert torch.equal(host, want)
