"""accumulate_lines on the GPU against the oracle (the reference CPU algorithm) and
the golden fixtures made by the reference itself: bit-exact where a term's value and
the merge are order-free (max in, max out; every single-line pixel), otherwise within
the sum-overlap tolerance (1e-5 relative + 1e-7 max_val absolute for float32)."""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from cbclib_v2_gb300 import _native, accumulate_lines, ndimage

pytestmark = pytest.mark.gpu

KERNELS = list(_native.KERNELS)
MODES = [('sum', 'sum'), ('max', 'sum'), ('sum', 'max'), ('max', 'max')]


def _tol(dtype, max_val):
    if dtype == np.float32:
        return dict(rtol=1e-5, atol=1e-7 * abs(max_val) + 1e-30)
    return dict(rtol=1e-12, atol=1e-14 * abs(max_val) + 1e-300)


def _case(seed, F=3, H=70, W=90, n=160, n_terms=25, dtype=np.float32):
    rng = np.random.default_rng(seed)
    p0 = rng.random((n, 2)) * [W, H]
    v = rng.normal(size=(n, 2))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    p1 = p0 + v * rng.uniform(2, 40, n)[:, None]
    lines = np.concatenate([p0, p1, rng.uniform(0.5, 5, (n, 1))], axis=1).astype(dtype)
    # terms gather nearby lines of one frame, so a term's lines overlap each other
    terms = rng.integers(0, n_terms, n)
    frames = rng.integers(0, F, n_terms)
    return (F, H, W), lines, terms, frames


def _run_both(shape, lines, terms, frames, max_val, kernel, iov, oov, dtype, out0=None):
    ref = np.zeros(shape, dtype) if out0 is None else out0.copy()
    oracle.accumulate_lines(ref, lines, terms, frames, max_val, kernel, iov, oov)
    got = torch.zeros(shape, dtype=torch.float32 if dtype == np.float32 else torch.float64,
                      device='cuda')
    if out0 is not None:
        got.copy_(torch.from_numpy(out0))
    accumulate_lines(got, torch.from_numpy(lines).cuda(), torch.from_numpy(terms).cuda(),
                     torch.from_numpy(frames).cuda(), max_val, kernel, iov, oov)
    return ref, got.cpu().numpy()


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("mode", MODES)
def test_random_float32(cuda, kernel, mode):
    shape, lines, terms, frames = _case(11)
    ref, got = _run_both(shape, lines, terms, frames, 3.0, kernel, *mode, np.float32)
    if mode == ('max', 'max'):
        assert np.array_equal(ref.view(np.uint32), got.view(np.uint32))
    else:
        np.testing.assert_allclose(got, ref, **_tol(np.float32, 3.0))


@pytest.mark.parametrize("kernel", ['gaussian', 'triangular'])
@pytest.mark.parametrize("mode", MODES)
def test_random_float64(cuda, kernel, mode):
    shape, lines, terms, frames = _case(12, dtype=np.float64)
    ref, got = _run_both(shape, lines, terms, frames, 2.0, kernel, *mode, np.float64)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("mode", MODES)
def test_negative_out_and_max_val(cuda, mode):
    """merges start from a zeroed term buffer: max merges lift negative pixels to 0"""
    shape, lines, terms, frames = _case(13, n=60)
    out0 = -np.random.default_rng(1).random(shape).astype(np.float32)
    for max_val in (1.5, -1.5):
        ref, got = _run_both(shape, lines, terms, frames, max_val, 'triangular', *mode,
                             np.float32, out0=out0)
        np.testing.assert_allclose(got, ref, **_tol(np.float32, max_val))


def test_golden_accumulate_fixtures(cuda, golden):
    cases = {k: c for k, c in golden.items() if c['kind'] == 'accumulate' and c['ndim'] == 2}
    assert cases
    for name, c in cases.items():
        dt = c['result'].dtype
        out = torch.zeros(tuple(c['result'].shape), dtype=torch.from_numpy(c['result']).dtype,
                          device='cuda')
        accumulate_lines(out, torch.from_numpy(c['lines']).cuda(), torch.from_numpy(c['terms']),
                         torch.from_numpy(c['frames']), c['max_val'], c['kernel'],
                         c['in_overlap'], c['out_overlap'])
        np.testing.assert_allclose(out.cpu().numpy(), c['result'], err_msg=name,
                                   **_tol(dt.type, c['max_val']))


def test_matches_draw_lines_for_single_line_terms(cuda):
    """one line per term, sum into out: the same pixels and values as draw_lines"""
    shape, lines, _, _ = _case(14, n=120)
    rng = np.random.default_rng(2)
    frames = rng.integers(0, shape[0], lines.shape[0])
    a = torch.zeros(shape, device='cuda')
    accumulate_lines(a, torch.from_numpy(lines).cuda(), np.arange(lines.shape[0]), frames,
                     2.0, 'gaussian', 'max', 'max')
    b = torch.zeros(shape, device='cuda')
    ndimage.draw_lines(b, torch.from_numpy(lines).cuda(), frames, 2.0, 'gaussian', 'max')
    assert torch.equal(a, b)


def test_host_arrays_and_int32_indices(cuda):
    shape, lines, terms, frames = _case(15, n=50)
    ref = np.zeros(shape, np.float32)
    oracle.accumulate_lines(ref, lines, terms, frames, 1.0, 'biweight', 'max', 'sum')
    out = np.zeros(shape, np.float32)
    accumulate_lines(out, lines, terms.astype(np.int32), frames.astype(np.int32), 1.0,
                     'biweight', 'max', 'sum')
    np.testing.assert_allclose(out, ref, **_tol(np.float32, 1.0))


def test_errors(cuda):
    shape, lines, terms, frames = _case(16, n=40, n_terms=5)
    out = torch.zeros(shape, device='cuda')
    bad_frames = frames.copy()
    bad_frames[2] = shape[0]
    with pytest.raises(IndexError, match=r"frames range \(\d+, 3\) is outside of \(0, 3\)"):
        accumulate_lines(out, lines, terms, bad_frames)
    bad_terms = terms.copy()
    bad_terms[7] = 5
    with pytest.raises(IndexError, match=r"Term index 5 is out of range \(0, 5\)"):
        accumulate_lines(out, lines, bad_terms, frames)
    with pytest.raises(ValueError, match="incompatible with number of lines"):
        accumulate_lines(out, lines, terms[:-1], frames)
    with pytest.raises(ValueError, match="Invalid overlap keyword"):
        accumulate_lines(out, lines, terms, frames, in_overlap='min')
    with pytest.raises(ValueError, match="kernel is missing"):
        accumulate_lines(out, lines, terms, frames, kernel='cosine')
    assert not out.any()                     # nothing drawn by the failed calls


def test_small_table_reports_capacity_and_draws_nothing(cuda):
    """through the C ABI: terms too large for shared memory (two of 300 lines) need the
    workspace table; a table too small for them sets CBC_ERR_CAPACITY, names a larger
    capacity and leaves out untouched"""
    n, n_terms = 600, 2
    shape, lines, terms, frames = _case(17, n=n, n_terms=n_terms)
    lib = _native.lib()
    out = torch.zeros(shape, device='cuda')
    ln = torch.from_numpy(lines).cuda()
    tm = torch.from_numpy(terms.astype(np.int64)).cuda()
    fr = torch.from_numpy(frames.astype(np.int64)).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    for cap in (0, 1024):
        ck = 16 * n + 1024
        nbytes = lib.cbc_accumulate_lines_workspace_size(n, n_terms, ck, cap, 4)
        ws = torch.empty(nbytes, dtype=torch.uint8, device='cuda')
        rc = lib.cbc_accumulate_lines_f32(out.data_ptr(), *shape, ln.data_ptr(), n,
                                          tm.data_ptr(), 8, fr.data_ptr(), 8, n_terms, 1.0,
                                          _native.KERNELS['rectangular'], 1, 0, ws.data_ptr(),
                                          nbytes, ck, cap, stream)
        assert rc == 0
        st = _native.Status()
        assert lib.cbc_read_status(ws.data_ptr(), ctypes.byref(st), stream) == 0
        assert st.has(_native.CBC_ERR_CAPACITY) and st.pairs_needed > cap
        assert not out.any()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("mode", [('max', 'sum'), ('sum', 'max')])
def test_mixed_term_sizes(cuda, dtype, mode):
    """terms of 1 to 400 lines in one call: small terms in one shared-memory pass,
    larger ones in several partitions, the largest through the workspace table (the
    host retries with the capacity the first call names)"""
    rng = np.random.default_rng(29)
    F, H, W = 2, 160, 200
    sizes = [1, 2, 3, 5, 8, 13, 40, 90, 400, 1, 7, 250]
    terms = np.repeat(np.arange(len(sizes)), sizes)
    n = terms.size
    frames = rng.integers(0, F, len(sizes))
    # each term's lines cluster around a centre, so they overlap one another
    centre = rng.random((len(sizes), 2)) * [W, H]
    p0 = centre[terms] + rng.normal(scale=25, size=(n, 2))
    v = rng.normal(size=(n, 2))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    p1 = p0 + v * rng.uniform(5, 60, n)[:, None]
    lines = np.concatenate([p0, p1, rng.uniform(0.5, 4, (n, 1))], axis=1).astype(dtype)
    perm = rng.permutation(n)
    lines, terms = lines[perm], terms[perm]
    ref, got = _run_both((F, H, W), lines, terms, frames, 2.0, 'triangular', *mode, dtype)
    np.testing.assert_allclose(got, ref, **_tol(dtype, 2.0))
    ws = next(w for k, w in ndimage._workspaces.items() if k[0] == 'accumulate')
    assert ws.capacity > 0                      # the largest terms went through the table
