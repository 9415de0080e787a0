"""Parity at the benchmark workloads' full sizes, against the oracle.

* Ragged stack, 256 frames of 1024x1024 with lognormal line counts (100 to 20,000
  per frame), triangular, sum: the CUDA-graph renderer's replay, compared on the
  frames with the fewest, the median and the most lines (sum within 1e-5 relative).
* Streak-fit stack, 32 frames of 2167x2070 with 5,000 biweight lines each, max: the
  packed (value, winner) forward that the fit loop runs, two frames bit for bit, the
  whole stack bit for bit against the plain max forward, and the packed loss step's
  gradient against the image path's.
* Detector stack, 64 frames of 2167x2070, gaussian, max: the whole stack drawn into
  page-locked host frames (the kernels combine the drawn pixels in place over the
  frames' device mapping), one frame bit for bit and the stack against the device
  path.
The seeds are the benchmark's, so these are the frames bench.py times.
"""
import os

import numpy as np
import pytest
import torch

import oracle
from cbclib_v2_gb300 import batch, draw_lines, fit, ndimage, workloads

pytestmark = pytest.mark.gpu

THREADS = max(1, len(os.sched_getaffinity(0)))


def sum_close(got, ref):
    bad = np.abs(got.astype(np.float64) - ref) > 1e-5 * np.abs(ref) + 1e-7
    assert not bad.any(), (int(bad.sum()), float(np.abs(got - ref).max()))


def test_ragged_stack_graph_replay(cuda, tmp_path, monkeypatch):
    monkeypatch.setenv('CBC_AUTOTUNE_CACHE', str(tmp_path / 'tune.json'))
    ls = workloads.ragged_stack(seed=3000)
    offs = ls.frame_offsets()
    counts = np.diff(offs)
    lines32 = ls.lines.astype(np.float32)
    r = batch.RaggedRenderer(ls.shape, offs, max_val=ls.max_val, kernel=ls.kernel,
                             overlap=ls.overlap, zero=True)
    r(torch.from_numpy(lines32).cuda())
    r.check()
    out = r.replay()                       # a second launch of the captured graph
    r.check()
    order = np.argsort(counts, kind='stable')
    picks = {'fewest': int(order[0]), 'median': int(order[len(order) // 2]),
             'most': int(order[-1])}
    for name, f in picks.items():
        sub = workloads.frames_subset(ls, [f])
        ref = oracle.draw_lines(np.zeros(sub.shape, np.float32), sub.lines.astype(np.float32),
                                sub.idxs, ls.max_val, ls.kernel, ls.overlap, THREADS)
        sum_close(out[f].cpu().numpy(), ref[0])


def test_fit_loop_stack_packed_forward(cuda):
    ls = workloads.fit_loop_stack(seed=4000)
    lines = torch.from_numpy(ls.lines.astype(np.float32)).cuda()
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).cuda()
    img = torch.empty(ls.shape, device='cuda')
    winner = ndimage.draw_lines_max_winner(img, lines, idxs, ls.max_val, ls.kernel)
    for f in (3, 29):
        sub = workloads.frames_subset(ls, [f])
        ref = oracle.draw_lines(np.zeros(sub.shape, np.float32), sub.lines.astype(np.float32),
                                sub.idxs, ls.max_val, ls.kernel, 'max', THREADS)
        assert np.array_equal(img[f].cpu().numpy(), ref[0]), f
    plain = torch.zeros(ls.shape, device='cuda')
    draw_lines(plain, lines, idxs, ls.max_val, ls.kernel, 'max')
    assert torch.equal(img, plain)
    drawn = img > 0
    assert int(drawn.sum()) > 0
    assert torch.all(winner[~drawn] == 0x7f7f7f7f)
    # the packed loss step (no frames) against the image path on the same lines
    target = torch.poisson(plain, generator=torch.Generator(device='cuda').manual_seed(4200))
    start = torch.from_numpy(workloads.perturbed(ls.lines, 4100, 1.0, 0.3)
                             .astype(np.float32)).cuda()
    image = torch.empty(ls.shape, device='cuda')
    want = fit.squared_loss_step(image, target, start, idxs, ls.max_val, ls.kernel, 'max')
    got = fit.squared_loss_step(None, target, start, idxs, ls.max_val, ls.kernel, 'max')
    torch.testing.assert_close(got, want, rtol=1e-5, atol=1e-3)


def test_detector_stack_pinned_host_frames(cuda):
    ls = workloads.detector_stack(seed=1000)
    lines32 = ls.lines.astype(np.float32)
    host = torch.zeros(ls.shape, dtype=torch.float32).pin_memory()
    draw_lines(host, torch.from_numpy(lines32).pin_memory(),
               torch.from_numpy(ls.idxs.astype(np.int32)).pin_memory(), ls.max_val, ls.kernel,
               ls.overlap)
    f = 37
    sub = workloads.frames_subset(ls, [f])
    ref = oracle.draw_lines(np.zeros(sub.shape, np.float32), sub.lines.astype(np.float32),
                            sub.idxs, ls.max_val, ls.kernel, ls.overlap, THREADS)
    assert np.array_equal(host[f].numpy(), ref[0])
    dev = torch.zeros(ls.shape, device='cuda')
    draw_lines(dev, torch.from_numpy(lines32).cuda(),
               torch.from_numpy(ls.idxs.astype(np.int32)).cuda(), ls.max_val, ls.kernel,
               ls.overlap)
    assert torch.equal(host, dev.cpu())
