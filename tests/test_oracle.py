"""The oracle (C restatement of the reference CPU rasteriser) is pinned: bit-exact on
every golden fixture produced by the reference itself, bit-exact against the
reference module on fresh random inputs when that module is built, and within the
reference test-suite's tolerance of its dense closed-form known answer."""
import numpy as np
import pytest

import oracle


def run_case(c):
    out = c['out0'].copy()
    if c['kind'] == 'draw':
        return oracle.draw_lines(out, c['lines'], c.get('idxs'), c['max_val'], c['kernel'],
                                 c['overlap'], 1)
    return oracle.accumulate_lines(out, c['lines'], c['terms'], c['frames'], c['max_val'],
                                   c['kernel'], c['in_overlap'], c['out_overlap'])


def test_golden_bit_exact(golden):
    bad = []
    for name, c in golden.items():
        got = run_case(c)
        if not np.array_equal(got.view(np.uint8), c['result'].view(np.uint8)):
            bad.append((name, int(np.sum(got != c['result']))))
    assert not bad, bad


def _random_lines(rng, n, H, W, ndim=2):
    sp = np.array([W, H] + ([H] if ndim == 3 else []), dtype=np.float64)[:ndim]
    p0 = rng.random((n, ndim)) * sp
    v = rng.normal(size=(n, ndim))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    p1 = p0 + v * rng.uniform(0, 60, n)[:, None]
    return np.concatenate([p0, p1, rng.uniform(0.3, 6, (n, 1))], axis=1)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("overlap", ['sum', 'max'])
def test_against_reference_module(dtype, overlap):
    ref = oracle.reference_module()
    if ref is None:
        pytest.skip("reference module not built (needs the reference checkout)")
    rng = np.random.default_rng(7)
    it = np.int32 if dtype == np.float32 else np.int64
    for kernel in oracle.KERNELS:
        lines = _random_lines(rng, 300, 70, 90).astype(dtype)
        idxs = rng.integers(0, 3, 300)
        a = np.full((3, 70, 90), 0.25, dtype)
        b = a.copy()
        ref.draw_lines(a, lines, idxs.astype(it), 1.5, kernel, overlap, 1)
        oracle.draw_lines(b, lines, idxs, 1.5, kernel, overlap, 1)
        assert np.array_equal(a, b), kernel


def _kernel_dense(name, x, sigma):
    """kernel table of the reference test (tests/draw_line_test.py:36-50)"""
    if name == 'biweight':
        return 0.9375 * np.clip(1 - (x / sigma)**2, 0, np.inf)**2
    if name == 'gaussian':
        return np.where(np.abs(x) < sigma, np.exp(-(3 * x / sigma)**2 / 2) / np.sqrt(2 * np.pi), 0)
    if name == 'parabolic':
        return 0.75 * np.clip(1 - (x / sigma)**2, 0, np.inf)
    if name == 'rectangular':
        return np.where(np.abs(x) < sigma, 1, 0)
    return np.clip(1 - np.abs(x / sigma), 0, np.inf)


def _project(lines, pts):
    """Lines.project (cbclib_v2/_src/streaks.py:52-59)"""
    ndim = lines.shape[-1] // 2
    pt0, pt1 = lines[..., :ndim], lines[..., ndim:2 * ndim]
    tau = pt1 - pt0
    center = 0.5 * (pt0 + pt1)
    r = pts - center
    r_tau = np.sum(tau * r, axis=-1) / np.sum(tau**2, axis=-1)
    r_tau = np.clip(r_tau[..., None], -0.5, 0.5)
    return tau * r_tau + center


@pytest.mark.parametrize("kernel", list(oracle.KERNELS))
@pytest.mark.parametrize("max_val", [1.0, 10.0])
def test_dense_known_answer(golden, kernel, max_val):
    """image_numpy of tests/draw_line_test.py:154-170 with check_close's float64
    tolerance (atol 1e-5, rtol 1e-4, cbclib_v2/_src/test_util.py:61-64)."""
    c = golden[f"reftest2d_float64_{kernel}_{max_val:g}_sum"]
    shape = tuple(c['shape'])
    lines, idxs, width = c['lines'], c['idxs'], 2.0
    pts = np.stack(np.meshgrid(*(np.arange(n) for n in shape[-2:]), indexing='ij')[::-1], -1)
    pts = pts[..., None, :].astype(np.float64)
    frames = []
    for f in range(int(np.prod(shape[:-2]))):
        lns = lines[idxs == f][:, :4]
        dist = pts - _project(lns, pts)
        img = max_val * _kernel_dense(kernel, np.sqrt(np.sum(dist**2, -1)), width)
        frames.append(np.sum(img, axis=-1))
    dense = np.stack(frames).reshape(shape)
    got = oracle.draw_lines(np.zeros(shape), lines, idxs, max_val, kernel, 'sum', 1)
    assert np.allclose(got, dense, rtol=1e-4, atol=1e-5)


def test_errors():
    out = np.zeros((2, 10, 10), np.float32)
    lines = np.array([[1, 1, 5, 5, 1.0]], np.float32)
    with pytest.raises(IndexError):
        oracle.draw_lines(out, lines, np.array([2]))
    with pytest.raises(ValueError):
        oracle.draw_lines(out, lines, None)          # 2 frames, 1 line, no idxs
    with pytest.raises(ValueError):
        oracle.draw_lines(out, lines, np.array([0]), kernel='box')
    with pytest.raises(ValueError):
        oracle.draw_lines(out, lines, np.array([0]), overlap='min')
