"""3-D lines (L = 7) into volumes on the GPU: draw_lines and accumulate_lines against the
oracle (the reference CPU algorithm's N = 3 walk) and the reference's own golden
fixtures.  max overlap is bit-exact; sum overlap differs only in the order in which a
voxel's contributions (including voxels the walk visits twice) are added."""
import numpy as np
import pytest
import torch

import oracle
from cbclib_v2_gb300 import _native, accumulate_lines, draw_lines

pytestmark = pytest.mark.gpu

KERNELS = list(_native.KERNELS)


def _tol(dtype, max_val):
    if dtype == np.float32:
        return dict(rtol=1e-5, atol=1e-6 * abs(max_val))
    return dict(rtol=1e-12, atol=1e-13 * abs(max_val))


def _lines3(seed, n, D, H, W, dtype, length=(2, 30), width=(0.4, 4)):
    rng = np.random.default_rng(seed)
    p0 = rng.random((n, 3)) * [W, H, D]
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    p1 = p0 + v * rng.uniform(*length, n)[:, None]
    return np.concatenate([p0, p1, rng.uniform(*width, (n, 1))], axis=1).astype(dtype)


def _torch_dtype(dtype):
    return torch.float32 if dtype == np.float32 else torch.float64


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("overlap", ['sum', 'max'])
@pytest.mark.parametrize("kernel", KERNELS)
def test_draw3d_random(cuda, dtype, overlap, kernel):
    F, D, H, W = 2, 18, 24, 30
    lines = _lines3(5, 60, D, H, W, dtype)
    idxs = np.random.default_rng(6).integers(0, F, lines.shape[0])
    ref = np.zeros((F, D, H, W), dtype)
    oracle.draw_lines(ref, lines, idxs, 2.5, kernel, overlap, 1)
    out = torch.zeros((F, D, H, W), dtype=_torch_dtype(dtype), device='cuda')
    draw_lines(out, torch.from_numpy(lines).cuda(), torch.from_numpy(idxs).cuda(), 2.5, kernel,
               overlap)
    got = out.cpu().numpy()
    if overlap == 'max' and not (dtype == np.float64 and kernel == 'gaussian'):
        assert np.array_equal(got, ref)
    else:
        np.testing.assert_allclose(got, ref, **_tol(dtype, 2.5))


def test_draw3d_golden(cuda, golden):
    cases = {k: c for k, c in golden.items() if c['kind'] == 'draw' and c['ndim'] == 3}
    assert cases
    for name, c in cases.items():
        res = c['result']
        out = torch.zeros(res.shape, dtype=torch.from_numpy(res).dtype, device='cuda')
        draw_lines(out, torch.from_numpy(c['lines']).cuda(),
                   None if c.get('idxs') is None else torch.from_numpy(c['idxs']).cuda(),
                   c['max_val'], c['kernel'], c['overlap'])
        np.testing.assert_allclose(out.cpu().numpy(), res, err_msg=name,
                                   **_tol(res.dtype.type, c['max_val']))


@pytest.mark.parametrize("mode", [('sum', 'sum'), ('max', 'sum'), ('sum', 'max'), ('max', 'max')])
@pytest.mark.parametrize("kernel", ['gaussian', 'rectangular', 'biweight'])
def test_accumulate3d_random(cuda, mode, kernel):
    F, D, H, W = 3, 16, 20, 26
    lines = _lines3(7, 70, D, H, W, np.float32)
    rng = np.random.default_rng(8)
    terms = rng.integers(0, 12, lines.shape[0])
    frames = rng.integers(0, F, 12)
    ref = np.zeros((F, D, H, W), np.float32)
    oracle.accumulate_lines(ref, lines, terms, frames, 1.5, kernel, *mode)
    out = torch.zeros((F, D, H, W), device='cuda')
    accumulate_lines(out, torch.from_numpy(lines).cuda(), terms, frames, 1.5, kernel, *mode)
    got = out.cpu().numpy()
    if mode == ('max', 'max'):
        assert np.array_equal(got, ref)
    else:
        np.testing.assert_allclose(got, ref, **_tol(np.float32, 1.5))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("mode", [('max', 'sum'), ('sum', 'max')])
def test_accumulate3d_mixed_term_sizes(cuda, dtype, mode):
    """terms of 1 to 500 lines in one call: the small ones in shared memory (in one or
    several partitions), the largest through the workspace table, whose capacity the
    first call names and the host retries with"""
    from cbclib_v2_gb300 import ndimage
    F, D, H, W = 2, 24, 28, 30
    sizes = [1, 3, 20, 500, 2, 60]
    rng = np.random.default_rng(31)
    terms = np.repeat(np.arange(len(sizes)), sizes)
    n = terms.size
    centre = rng.random((len(sizes), 3)) * [W, H, D]
    p0 = centre[terms] + rng.normal(scale=5, size=(n, 3))
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    p1 = p0 + v * rng.uniform(4, 25, n)[:, None]
    lines = np.concatenate([p0, p1, rng.uniform(0.7, 2.5, (n, 1))], axis=1).astype(dtype)
    perm = rng.permutation(n)
    lines, terms = lines[perm], terms[perm]
    frames = rng.integers(0, F, len(sizes))
    ref = np.zeros((F, D, H, W), dtype)
    oracle.accumulate_lines(ref, lines, terms, frames, 1.5, 'gaussian', *mode)
    out = torch.zeros((F, D, H, W), dtype=torch.from_numpy(ref).dtype, device='cuda')
    accumulate_lines(out, torch.from_numpy(lines).cuda(), terms, frames, 1.5, 'gaussian', *mode)
    np.testing.assert_allclose(out.cpu().numpy(), ref, **_tol(dtype, 1.5))
    ws = next(w for k, w in ndimage._workspaces.items() if k[0] == 'accumulate3d')
    assert ws.capacity > 0                      # the largest terms went through the table


def test_accumulate3d_golden(cuda, golden):
    """the reference rotomap's form: gaussian, max within terms, sum across terms"""
    cases = {k: c for k, c in golden.items() if c['kind'] == 'accumulate' and c['ndim'] == 3}
    assert cases
    for name, c in cases.items():
        res = c['result']
        out = torch.zeros(res.shape, dtype=torch.from_numpy(res).dtype, device='cuda')
        accumulate_lines(out, torch.from_numpy(c['lines']).cuda(), c['terms'], c['frames'],
                         c['max_val'], c['kernel'], c['in_overlap'], c['out_overlap'])
        np.testing.assert_allclose(out.cpu().numpy(), res, err_msg=name,
                                   **_tol(res.dtype.type, c['max_val']))


def test_draw3d_single_volume_and_errors(cuda):
    D, H, W = 12, 14, 16
    lines = _lines3(9, 20, D, H, W, np.float32)
    ref = np.zeros((D, H, W), np.float32)
    oracle.draw_lines(ref, lines, None, 1.0, 'triangular', 'sum', 1)
    out = torch.zeros((D, H, W), device='cuda')
    draw_lines(out, lines, None, 1.0, 'triangular', 'sum')
    np.testing.assert_allclose(out.cpu().numpy(), ref, **_tol(np.float32, 1.0))
    with pytest.raises(IndexError):
        draw_lines(torch.zeros((2, D, H, W), device='cuda'), lines, np.full(20, 2), 1.0)
    with pytest.raises(ValueError, match="do not match the line size"):
        draw_lines(torch.zeros((H, W), device='cuda'), lines)
