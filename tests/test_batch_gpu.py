"""Ragged stacks: CSR frame offsets, the CUDA-graph renderer and the autotuner, all
checked against the oracle (max overlap bit-exact, sum within 1e-5 relative)."""
import numpy as np
import pytest
import torch

import oracle
from cbclib_v2_gb300 import autotune, batch, ndimage, workloads

pytestmark = pytest.mark.gpu


def small_ragged(seed=0, F=6, H=120, W=150):
    rng = np.random.default_rng(seed)
    counts = np.array([40, 0, 3, 120, 15, 60])[:F]
    n = int(counts.sum())
    p0 = rng.random((n, 2)) * [W, H]
    ang = rng.random(n) * 2 * np.pi
    L = rng.uniform(5, 60, n)
    lines = np.c_[p0, p0 + L[:, None] * np.c_[np.cos(ang), np.sin(ang)], rng.uniform(1, 4, n)]
    offs = np.r_[0, np.cumsum(counts)].astype(np.int64)
    idxs = np.repeat(np.arange(F), counts)
    return lines.astype(np.float32), offs, idxs, (F, H, W)


def check(got, ref, overlap):
    if overlap == 'max':
        assert np.array_equal(got, ref)
    else:
        assert np.all(np.abs(got - ref) <= 1e-5 * np.abs(ref) + 1e-7)


@pytest.mark.parametrize("overlap", ['sum', 'max'])
def test_csr_matches_oracle(cuda, overlap):
    lines, offs, idxs, shape = small_ragged()
    ref = oracle.draw_lines(np.zeros(shape, np.float32), lines, idxs, 1.5, 'triangular', overlap, 1)
    out = torch.zeros(shape, device='cuda')
    ndimage.draw_lines_csr(out, torch.tensor(lines, device='cuda'), torch.tensor(offs), 1.5,
                           'triangular', overlap)
    check(out.cpu().numpy(), ref, overlap)


def test_csr_rejects_bad_offsets(cuda):
    lines, offs, _, shape = small_ragged()
    out = torch.full(shape, 2.0, device='cuda')
    bad = offs.copy()
    bad[3], bad[4] = bad[4], bad[3]              # decreasing
    with pytest.raises(IndexError):
        ndimage.draw_lines_csr(out, torch.tensor(lines, device='cuda'), torch.tensor(bad))
    bad = offs.copy()
    bad[-1] -= 1                                  # does not end at n_lines
    with pytest.raises(IndexError):
        ndimage.draw_lines_csr(out, torch.tensor(lines, device='cuda'), torch.tensor(bad))
    assert float(out.min()) == 2.0 and float(out.max()) == 2.0


@pytest.mark.parametrize("overlap", ['sum', 'max'])
def test_graph_renderer_replays(cuda, overlap):
    lines, offs, idxs, shape = small_ragged(seed=3)
    r = batch.RaggedRenderer(shape, offs, max_val=1.0, kernel='biweight', overlap=overlap,
                             zero=True)
    for trial in range(2):
        ln = lines + (0 if trial == 0 else np.float32(0.3))
        got = r(torch.tensor(ln, device='cuda')).cpu().numpy()
        r.check()
        ref = oracle.draw_lines(np.zeros(shape, np.float32), ln, idxs, 1.0, 'biweight', overlap, 1)
        check(got, ref, overlap)
    assert r.timings, "the renderer autotunes its configuration"


def test_per_frame_launches_agree(cuda):
    lines, offs, idxs, shape = small_ragged(seed=4)
    a = torch.zeros(shape, device='cuda')
    b = torch.zeros(shape, device='cuda')
    t = torch.tensor(lines, device='cuda')
    ndimage.draw_lines_csr(a, t, torch.tensor(offs), 1.0, 'gaussian', 'max')
    batch.render_per_frame(b, t, offs, 1.0, 'gaussian', 'max')
    assert torch.equal(a, b)


def test_autotune_picks_and_caches(cuda, tmp_path, monkeypatch):
    monkeypatch.setenv('CBC_AUTOTUNE_CACHE', str(tmp_path / 'tune.json'))
    ls = workloads.ragged_stack(seed=1, F=8, H=256, W=256, median=400)
    out = torch.zeros(ls.shape, device='cuda')
    lines = torch.tensor(ls.lines, dtype=torch.float32, device='cuda')
    idxs = torch.tensor(ls.idxs, device='cuda')
    best, timings = autotune.tune(out, lines, idxs, 1.0, ls.kernel, 'max')
    assert len(timings) == len(autotune.candidates())
    assert float(out.abs().sum()) == 0.0
    key = autotune.workload_key(out.shape, out.dtype, ls.kernel, 'max', lines.shape[0])
    assert autotune.lookup(key) is not None
    a = torch.zeros(ls.shape, device='cuda')
    ndimage.draw_lines(a, lines, idxs, 1.0, ls.kernel, 'max')       # uses the cached choice
    ref = oracle.draw_lines(np.zeros(ls.shape, np.float32), ls.lines.astype(np.float32),
                            ls.idxs, 1.0, ls.kernel, 'max', 4)
    assert np.array_equal(a.cpu().numpy(), ref)
