"""GPU parity of cbclib_v2_gb300.draw_lines with the reference CPU path.

Gates (the tolerances are written here):
  * max overlap: bit-exact against the reference (golden fixtures) and the oracle;
  * sum overlap: every pixel within |d| <= 1e-5 |ref| + 1e-7 max_val of the reference
    (contributions are bit-identical; only the order of additions differs);
  * rectangular profile with unit contributions: bit-exact for sum too (exact sums).
"""
import zlib

import numpy as np
import pytest
import torch

import oracle
from cbclib_v2_gb300 import _native, device, draw_lines, ndimage, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True, params=['tiles', 'lines'])
def strategy(request):
    """every test runs under both render strategies"""
    code = {'tiles': _native.STRATEGY_TILES, 'lines': _native.STRATEGY_LINES}[request.param]
    with ndimage.tuning(strategy=code):
        yield request.param

SUM_RTOL = 1e-5
SUM_ATOL = 1e-7


def assert_parity(got, ref, overlap, max_val=1.0, kernel=None):
    got = np.asarray(got)
    if got.dtype == np.float64 and kernel == 'gaussian':
        # float64 gaussian: the device's double exp may differ from the host libm's by
        # an ulp, so both overlaps are compared to a few ulp of float64
        assert np.allclose(got, ref, rtol=1e-14, atol=1e-15 * abs(max_val))
        return
    if overlap == 'max':
        bad = np.sum(got.view(np.uint8).reshape(got.shape + (-1,)) !=
                     ref.view(np.uint8).reshape(ref.shape + (-1,)))
        assert bad == 0, f"{int(np.sum(got != ref))} pixels differ (max overlap must be bit-exact)"
    else:
        tol = SUM_RTOL * np.abs(ref) + SUM_ATOL * abs(max_val)
        err = np.abs(got.astype(np.float64) - ref)
        assert np.all(err <= tol), f"max err {err.max()} at {np.unravel_index(err.argmax(), err.shape)}"


def gpu_draw(c, **kw):
    out = torch.from_numpy(c['out0'].copy()).cuda()
    idxs = c.get('idxs')
    res = draw_lines(out, torch.from_numpy(c['lines']).cuda(),
                     None if idxs is None else torch.from_numpy(np.asarray(idxs)).cuda(),
                     c['max_val'], c['kernel'], c['overlap'], **kw)
    assert res is out
    return out.cpu().numpy()


def test_golden_fixtures(cuda, golden):
    n, bad = 0, []
    for name, c in golden.items():
        if c['kind'] != 'draw' or c['ndim'] != 2:
            continue
        try:
            assert_parity(gpu_draw(c), c['result'], c['overlap'], c['max_val'], c['kernel'])
        except AssertionError as e:
            bad.append(f"{name}: {e}")
        n += 1
    assert not bad, bad
    assert n > 60


def _rand_lines(rng, n, F, H, W, lmax=80.0, wmin=0.3, wmax=6.0):
    p0 = rng.random((n, 2)) * np.array([W, H])
    ang = rng.random(n) * 2 * np.pi
    L = rng.random(n) * lmax
    p1 = p0 + L[:, None] * np.stack([np.cos(ang), np.sin(ang)], -1)
    w = rng.uniform(wmin, wmax, n)
    return np.c_[p0, p1, w], rng.integers(0, F, n)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("kernel", list(oracle.KERNELS))
@pytest.mark.parametrize("overlap", ['sum', 'max'])
def test_random_vs_oracle(cuda, dtype, kernel, overlap):
    rng = np.random.default_rng(zlib.crc32(f'{np.dtype(dtype).name}{kernel}{overlap}'.encode()))
    F, H, W = 3, 150, 211
    lines, idxs = _rand_lines(rng, 700, F, H, W)
    lines = lines.astype(dtype)
    out0 = (rng.random((F, H, W)) * 0.5).astype(dtype)
    ref = oracle.draw_lines(out0.copy(), lines, idxs, 1.7, kernel, overlap, 1)
    for idt in (torch.int32, torch.int64):
        out = torch.from_numpy(out0.copy()).cuda()
        draw_lines(out, torch.from_numpy(lines).cuda(), torch.from_numpy(idxs).to(idt).cuda(),
                   1.7, kernel, overlap)
        assert_parity(out.cpu().numpy(), ref, overlap, 1.7, kernel)


@pytest.mark.parametrize("tile", [(16, 16), (32, 8), (64, 64), (128, 32), (256, 4)])
def test_tile_shapes(cuda, tile):
    from cbclib_v2_gb300 import _native, ndimage
    rng = np.random.default_rng(3)
    F, H, W = 2, 97, 301
    lines, idxs = _rand_lines(rng, 500, F, H, W, lmax=150, wmax=12)
    lines = lines.astype(np.float32)
    for overlap in ('sum', 'max'):
        ref = oracle.draw_lines(np.zeros((F, H, W), np.float32), lines, idxs, 1.0, 'biweight',
                                overlap, 1)
        out = torch.zeros((F, H, W), dtype=torch.float32, device='cuda')
        t = _native.Tuning(tile[0], tile[1], 8, 0, _native.STRATEGY_TILES, 0)
        ndimage._draw_lines_cuda(out, torch.from_numpy(lines).cuda(), torch.from_numpy(idxs).cuda(),
                                 1.0, 0, _native.OVERLAPS[overlap], tuning=t)
        assert_parity(out.cpu().numpy(), ref, overlap)


def test_single_frame_workload_exact(cuda):
    """The 512x512, 1,000-segment rectangular/sum workload: unit contributions sum
    exactly, so the result is bit-exact in any order."""
    ls = workloads.single_frame(seed=5)
    lines = ls.lines.astype(np.float32)
    ref = oracle.draw_lines(np.zeros(ls.shape, np.float32), lines, None, 1.0, ls.kernel,
                            ls.overlap, 1)
    out = torch.zeros(ls.shape, dtype=torch.float32, device='cuda')
    draw_lines(out, torch.from_numpy(lines).cuda(), None, 1.0, ls.kernel, ls.overlap)
    assert np.array_equal(out.cpu().numpy(), ref)


def test_detector_frames_exact(cuda):
    """Two frames of the 64 x 2167 x 2070 gaussian/max workload against the oracle."""
    ls = workloads.detector_stack(seed=1, F=64)
    sub = workloads.frames_subset(ls, [5, 40])
    lines = sub.lines.astype(np.float32)
    ref = oracle.draw_lines(np.zeros(sub.shape, np.float32), lines, sub.idxs, 1.0, sub.kernel,
                            sub.overlap, 4)
    out = torch.zeros(sub.shape, dtype=torch.float32, device='cuda')
    draw_lines(out, torch.from_numpy(lines).cuda(), torch.from_numpy(sub.idxs.astype(np.int32)).cuda(),
               1.0, sub.kernel, sub.overlap)
    assert_parity(out.cpu().numpy(), ref, 'max')


def test_full_detector_stack_properties(cuda):
    """Full-size workload: max overlap is order-independent, so two runs agree bit for
    bit, and frames checked on the CPU match exactly."""
    ls = workloads.detector_stack(seed=2)
    lines = torch.from_numpy(ls.lines.astype(np.float32)).cuda()
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).cuda()
    a = torch.zeros(ls.shape, dtype=torch.float32, device='cuda')
    b = torch.zeros(ls.shape, dtype=torch.float32, device='cuda')
    draw_lines(a, lines, idxs, 1.0, ls.kernel, ls.overlap)
    draw_lines(b, lines, idxs, 1.0, ls.kernel, ls.overlap)
    assert torch.equal(a, b)
    assert float(a.max()) <= 0.3989423 and float(a.min()) == 0.0
    f = 63
    sub = workloads.frames_subset(ls, [f])
    ref = oracle.draw_lines(np.zeros(sub.shape, np.float32), sub.lines.astype(np.float32),
                            sub.idxs, 1.0, ls.kernel, ls.overlap, 4)
    assert_parity(a[f:f + 1].cpu().numpy(), ref, 'max')


def test_accumulates_into_out(cuda):
    rng = np.random.default_rng(9)
    lines, idxs = _rand_lines(rng, 50, 1, 40, 40)
    lines = lines.astype(np.float32)
    out0 = np.full((40, 40), 1.0, np.float32)
    ref = oracle.draw_lines(out0.copy(), lines, None, 1.0, 'rectangular', 'sum', 1)
    out = torch.from_numpy(out0.copy()).cuda()
    draw_lines(out, torch.from_numpy(lines).cuda())
    assert np.array_equal(out.cpu().numpy(), ref)
    assert float(out.min()) == 1.0


def test_empty_and_degenerate(cuda):
    out = torch.zeros((3, 16, 22), device='cuda', dtype=torch.float64)
    draw_lines(out, torch.zeros((0, 5), dtype=torch.float64))
    assert float(out.sum()) == 0.0
    rng = np.random.default_rng(4)
    lines, idxs = _rand_lines(rng, 40, 3, 16, 22)
    for w in (0.0, -1.0):
        ln = lines.copy()
        ln[:, 4] = w
        for kernel in oracle.KERNELS:
            draw_lines(out, ln, idxs, kernel=kernel)
            assert float(out.sum()) == 0.0
    bad = lines.copy()
    bad[::3, 0] = np.nan
    bad[1::3, 4] = np.inf
    ref = oracle.draw_lines(np.zeros((3, 16, 22)), bad, idxs, 1.0, 'biweight', 'max', 1)
    out.zero_()
    draw_lines(out, bad, idxs, 1.0, 'biweight', 'max')
    assert np.array_equal(out.cpu().numpy(), ref)


def test_errors_leave_out_untouched(cuda):
    out = torch.full((2, 10, 12), 3.0, device='cuda')
    lines = torch.tensor([[1, 1, 8, 8, 2.0], [2, 9, 9, 2, 1.0]], device='cuda')
    with pytest.raises(IndexError, match=r"\(0, 2\)"):
        draw_lines(out, lines, torch.tensor([0, 2], device='cuda'))
    with pytest.raises(IndexError):
        draw_lines(out, lines, torch.tensor([-1, 0], device='cuda'))
    assert float(out.min()) == 3.0 and float(out.max()) == 3.0
    with pytest.raises(ValueError):
        draw_lines(out, lines[:1], torch.tensor([0, 1], device='cuda'))   # size mismatch
    with pytest.raises(ValueError):
        draw_lines(out, lines[:1])                                       # 2 frames, 1 line
    with pytest.raises(RuntimeError):
        draw_lines(out, torch.zeros((3, 4), device='cuda'))              # L = 4


def test_host_arrays_and_layouts(cuda):
    rng = np.random.default_rng(12)
    lines, idxs = _rand_lines(rng, 200, 4, 30, 50)
    lines = lines.astype(np.float32)
    ref = oracle.draw_lines(np.zeros((4, 30, 50), np.float32), lines, idxs, 2.0, 'triangular',
                            'max', 1)
    host = np.zeros((4, 30, 50), np.float32)
    with device.context('cuda'):
        res = draw_lines(host, lines, idxs, 2.0, 'triangular', 'max')
    assert res is host and np.array_equal(host, ref)
    # non-contiguous CUDA output (a strided view) is updated in place
    big = torch.zeros((4, 30, 100), device='cuda')
    view = big[:, :, ::2]
    draw_lines(view, lines, idxs, 2.0, 'triangular', 'max')
    assert np.array_equal(view.cpu().numpy(), ref)
    assert float(big[:, :, 1::2].abs().sum()) == 0.0
    # leading frame dimensions are flattened like the reference
    out4 = torch.zeros((2, 2, 30, 50), device='cuda')
    draw_lines(out4, lines, idxs, 2.0, 'triangular', 'max')
    assert np.array_equal(out4.cpu().numpy().reshape(4, 30, 50), ref)


def test_capacity_growth(cuda):
    """Long thick lines produce many (line, tile) pairs; the first call overflows the
    initial pair capacity, draws nothing, and the retry draws everything."""
    from cbclib_v2_gb300 import ndimage
    ndimage._workspaces.clear()
    rng = np.random.default_rng(21)
    lines, idxs = _rand_lines(rng, 60, 1, 900, 900, lmax=1200, wmin=30, wmax=80)
    lines = lines.astype(np.float32)
    ref = oracle.draw_lines(np.zeros((900, 900), np.float32), lines, None, 1.0, 'parabolic',
                            'max', 4)
    out = torch.zeros((900, 900), device='cuda')
    draw_lines(out, lines, None, 1.0, 'parabolic', 'max')
    assert np.array_equal(out.cpu().numpy(), ref)
