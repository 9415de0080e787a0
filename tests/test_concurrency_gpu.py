"""Calls from several host threads, each on its own stream, and index layouts: the
library keeps a workspace per (device, stream, thread), so concurrent calls give the
results of sequential ones; the frame index order and width do not change a
max-overlap result (bit-exact)."""
import threading

import numpy as np
import pytest
import torch

from cbclib_v2_gb300 import draw_lines, fit, ndimage, workloads

pytestmark = pytest.mark.gpu


def stack(seed, F=6, H=300, W=280, per_frame=300):
    ls = workloads.fit_loop_stack(seed=seed, F=F, H=H, W=W, per_frame=per_frame)
    return (torch.from_numpy(ls.lines.astype(np.float32)).cuda(),
            torch.from_numpy(ls.idxs.astype(np.int32)).cuda(), ls)


def test_threads_on_own_streams_match_sequential(cuda):
    jobs = [stack(100 + k) for k in range(4)]
    want = []
    for lines, idxs, ls in jobs:
        out = torch.zeros(ls.shape, device='cuda')
        draw_lines(out, lines, idxs, ls.max_val, 'gaussian', 'max')
        want.append(out)
    got = [None] * len(jobs)
    errors = []

    def work(k):
        try:
            lines, idxs, ls = jobs[k]
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                for _ in range(5):               # repeated calls reuse the thread's workspace
                    out = torch.zeros(ls.shape, device='cuda')
                    draw_lines(out, lines, idxs, ls.max_val, 'gaussian', 'max')
            s.synchronize()
            got[k] = out
        except BaseException as e:         # reported in the main thread
            errors.append(e)

    threads = [threading.Thread(target=work, args=(k,)) for k in range(len(jobs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for g, w in zip(got, want):
        assert torch.equal(g, w)


def test_fused_loss_steps_from_threads(cuda):
    """the packed scratch of the fused loss step is per (device, stream, thread)"""
    jobs = [stack(200 + k, F=3) for k in range(3)]
    targets = [torch.rand(ls.shape, device='cuda') * 3 for _, _, ls in jobs]
    want = [fit.squared_loss_step(None, t, l, i, ls.max_val, ls.kernel, 'max')
            for (l, i, ls), t in zip(jobs, targets)]
    got = [None] * len(jobs)
    errors = []

    def work(k):
        try:
            l, i, ls = jobs[k]
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                for _ in range(4):
                    g = fit.squared_loss_step(None, targets[k], l, i, ls.max_val, ls.kernel, 'max')
            s.synchronize()
            got[k] = g
        except BaseException as e:
            errors.append(e)

    threads = [threading.Thread(target=work, args=(k,)) for k in range(len(jobs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for g, w in zip(got, want):
        torch.testing.assert_close(g, w, rtol=1e-5, atol=1e-4)


def test_index_order_and_width_do_not_matter(cuda):
    lines, idxs, ls = stack(300)
    ref = torch.zeros(ls.shape, device='cuda')
    draw_lines(ref, lines, idxs, ls.max_val, 'biweight', 'max')
    perm = torch.from_numpy(np.random.default_rng(301).permutation(lines.shape[0])).cuda()
    for ix in (idxs[perm].to(torch.int64), idxs[perm]):
        out = torch.zeros(ls.shape, device='cuda')
        draw_lines(out, lines[perm], ix, ls.max_val, 'biweight', 'max')
        assert torch.equal(out, ref)
    out = torch.zeros(ls.shape, device='cuda')
    draw_lines(out, lines, idxs.to(torch.int64), ls.max_val, 'biweight', 'max')
    assert torch.equal(out, ref)
