"""Streak-fit loop (fit.fit_lines): Adam on the line parameters through the forward and
adjoint kernels recovers lines perturbed by about a pixel."""
import numpy as np
import pytest
import torch

from cbclib_v2_gb300 import draw_lines, fit, workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("overlap", ['max', 'sum'])
def test_fit_recovers_perturbed_lines(cuda, overlap):
    ls = workloads.fit_loop_stack(seed=7, F=2, H=256, W=256, per_frame=60)
    truth = torch.from_numpy(ls.lines.astype(np.float32)).cuda()
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).cuda()
    target = torch.zeros(ls.shape, device='cuda')
    draw_lines(target, truth, idxs, ls.max_val, ls.kernel, overlap)
    start = torch.from_numpy(workloads.perturbed(ls.lines, 8, 1.0, 0.3).astype(np.float32)).cuda()
    res = fit.fit_lines(target, start, idxs, max_val=ls.max_val, kernel=ls.kernel,
                        overlap=overlap, steps=150, lr=0.05)
    rms0 = float((start - truth)[:, :4].pow(2).mean().sqrt())
    rms1 = float((res.lines - truth)[:, :4].pow(2).mean().sqrt())
    assert res.losses[-1] < 0.2 * res.losses[0]
    assert rms1 < 0.5 * rms0
    assert torch.all(res.lines[:, 4] >= 0.5)


def test_fit_rejects_host_target():
    with pytest.raises(ValueError):
        fit.fit_lines(torch.zeros(1, 8, 8), torch.zeros(1, 5))
