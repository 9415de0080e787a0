"""The adjoint's frame-shaped arguments are checked before any device work: a buffer
with fewer elements than the frames would let the kernels read or write past it."""
import pytest
import torch

from cbclib_v2_gb300 import autograd


def test_frame_shaped_arguments_must_cover_the_frames():
    g = torch.zeros((2, 30, 40))
    lines = torch.zeros((3, 5))
    small = torch.zeros((2, 30, 39))
    with pytest.raises(ValueError, match='image'):
        autograd.lines_backward(g, lines, None, 1.0, 'biweight', 'max', image=small)
    with pytest.raises(ValueError, match='out0'):
        autograd.lines_backward(g, lines, None, 1.0, 'biweight', 'max', image=g, out0=small)
    with pytest.raises(ValueError, match='target'):
        autograd.squared_loss_backward(g, small, lines, None, 1.0, 'biweight', 'sum')


def test_winner_buffer_is_checked():
    g = torch.zeros((2, 30, 40))
    lines = torch.zeros((3, 5))
    for bad in (torch.zeros((2, 30, 40), dtype=torch.int64),
                torch.zeros((2, 30, 39), dtype=torch.int32),
                torch.zeros((2, 40, 30), dtype=torch.int32).transpose(1, 2)):
        with pytest.raises(ValueError, match='winner'):
            autograd.lines_backward(g, lines, None, 1.0, 'biweight', 'max', image=g, winner=bad)
