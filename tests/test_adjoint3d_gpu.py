"""The 3-D adjoint (gradient of draw_lines for lines (N, 7) into volumes with respect
to x0, y0, z0, x1, y1, z1, width) against finite differences of the float64 oracle
forward, for L = sum((I - T)^2) with a fixed target T.

The reference value is Richardson-extrapolated central differences: R(h) =
2 D(h / 2) - D(h) from steps h = 1e-3 and 5e-4 px, and again from 5e-4 and 2.5e-4 px.
Plain central differences converge only linearly here: the biweight is C1 but its
second derivative jumps at the support edge, and a 3-D tube has many voxels within a
step of that edge (at h = 1e-3 px, D(h) is off by up to 3e-4 relative).  A parameter
whose two extrapolations disagree (a step that changes how often the walk visits a
voxel: the 3-D walk visits some voxels twice and sum overlap adds each visit, or a
voxel entering the walk) is left out; the test checks that nearly all remain.

Gate: relative error <= 1e-4 (float64 adjoint) on every kept parameter whose gradient
exceeds 1% of the largest, and on the kept gradient vector in the 2-norm; the float32
adjoint on the 2-norm.  For max overlap the lines are kept apart so that no voxel
switches winner."""
import numpy as np
import pytest
import torch

import oracle
from cbclib_v2_gb300 import _native, autograd, draw_lines

pytestmark = pytest.mark.gpu

STEP = 1e-3
RTOL = 1e-4
SHAPE = (2, 18, 22, 26)


def loss(lines, idxs, target, kernel, overlap, max_val):
    img = oracle.draw_lines(np.zeros(SHAPE), lines, idxs, max_val, kernel, overlap, 1)
    return float(np.sum((img - target) ** 2))


def fd(lines, idxs, target, kernel, overlap, max_val, h):
    g = np.zeros_like(lines)
    for i in range(lines.shape[0]):
        for k in range(7):
            lp, lm = lines.copy(), lines.copy()
            lp[i, k] += h
            lm[i, k] -= h
            g[i, k] = (loss(lp, idxs, target, kernel, overlap, max_val) -
                       loss(lm, idxs, target, kernel, overlap, max_val)) / (2 * h)
    return g


def adjoint(lines, idxs, target, kernel, overlap, max_val, dtype):
    ln = torch.tensor(lines, dtype=dtype, device='cuda', requires_grad=True)
    img = autograd.draw_lines_fn(ln, torch.tensor(idxs, device='cuda'), shape=SHAPE,
                                 max_val=max_val, kernel=kernel, overlap=overlap)
    ((img - torch.tensor(target, dtype=dtype, device='cuda')) ** 2).sum().backward()
    return ln.grad.double().cpu().numpy(), img.detach().double().cpu().numpy()


def extrapolated(lines, idxs, target, kernel, overlap, max_val):
    """(R(h / 2), kept): Richardson-extrapolated central differences and the parameters
    whose extrapolations from (h, h / 2) and (h / 2, h / 4) agree"""
    d1, d2, d4 = (fd(lines, idxs, target, kernel, overlap, max_val, STEP / m) for m in (1, 2, 4))
    r1, r2 = 2 * d2 - d1, 2 * d4 - d2
    keep = np.abs(r1 - r2) <= 2e-5 * np.abs(r2) + 1e-7 * np.abs(r2).max()
    return r2, keep


def errors(got, want, keep):
    big = keep & (np.abs(want) > 0.01 * np.abs(want[keep]).max())
    per = (np.abs(got - want)[big] / np.abs(want)[big]).max()
    norm = np.linalg.norm((got - want)[keep]) / np.linalg.norm(want[keep])
    return per, norm


def random_lines(rng, n):
    p0 = rng.uniform([4, 4, 4], [22, 18, 14], (n, 3))
    v = rng.normal(size=(n, 3))
    v *= rng.uniform(3, 9, (n, 1)) / np.linalg.norm(v, axis=1, keepdims=True)
    return np.c_[p0, p0 + v, rng.uniform(1.6, 3.2, n)]


def separated_lines(rng):
    rows = []
    for cx, cy in ((6.5, 6.0), (19.5, 6.0), (6.5, 16.0), (19.5, 16.0)):
        c = np.array([cx, cy, 9.0])
        v = rng.normal(size=3)
        v *= rng.uniform(2.5, 4.5) / np.linalg.norm(v)
        rows.append([*(c - v), *(c + v), rng.uniform(1.5, 2.2)])
    return np.array(rows)


@pytest.mark.parametrize("overlap", ['sum', 'max'])
def test_gradient3d_matches_fp64_finite_differences(cuda, overlap):
    rng = np.random.default_rng(51 if overlap == 'sum' else 52)
    if overlap == 'sum':
        lines = random_lines(rng, 6)
        idxs = rng.integers(0, SHAPE[0], 6)
    else:
        lines = separated_lines(rng)
        idxs = np.array([0, 1, 1, 0])
    target = rng.random(SHAPE) * 0.5
    kernel, max_val = 'biweight', 1.3
    want, keep = extrapolated(lines, idxs, target, kernel, overlap, max_val)
    assert keep.mean() >= 0.8, keep.mean()
    got, img = adjoint(lines, idxs, target, kernel, overlap, max_val, torch.float64)
    ref = oracle.draw_lines(np.zeros(SHAPE), lines, idxs, max_val, kernel, overlap, 1)
    assert np.allclose(img, ref, rtol=1e-13, atol=1e-14)
    per, norm = errors(got, want, keep)
    print(f"3-D float64 adjoint, {overlap}: per parameter {per:.3e}, 2-norm {norm:.3e}, "
          f"{int(keep.sum())} of {keep.size} parameters smooth")
    assert per <= RTOL and norm <= RTOL, (per, norm)
    got32, _ = adjoint(lines, idxs, target, kernel, overlap, max_val, torch.float32)
    per32, norm32 = errors(got32, want, keep)
    print(f"3-D float32 adjoint, {overlap}: per parameter {per32:.3e}, 2-norm {norm32:.3e}")
    assert norm32 <= RTOL, (per32, norm32)


@pytest.mark.parametrize("kernel", ['gaussian', 'parabolic', 'triangular', 'rectangular'])
def test_gradient3d_other_profiles_sum_and_max(cuda, kernel):
    """the other profiles against finite differences where the loss is smooth (the
    gaussian jumps at its support edge, rectangular is flat: its gradient is zero)"""
    rng = np.random.default_rng(53)
    lines = separated_lines(rng)
    idxs = np.array([0, 1, 1, 0])
    target = rng.random(SHAPE) * 0.5
    for overlap in ('sum', 'max'):
        got, _ = adjoint(lines, idxs, target, kernel, overlap, 1.1, torch.float64)
        if kernel == 'rectangular':
            assert np.all(got == 0)
            continue
        want, keep = extrapolated(lines, idxs, target, kernel, overlap, 1.1)
        assert keep.mean() >= 0.5, keep.mean()
        per, norm = errors(got, want, keep)
        assert norm <= 1e-3, (kernel, overlap, per, norm)


def test_winners3d_and_out0_gradient(cuda):
    """max overlap with a non-zero base: the winners come back as line indices or
    NO_WINNER, and d/d(out0) is the upstream gradient exactly where no line won"""
    rng = np.random.default_rng(54)
    lines = separated_lines(rng)
    idxs = np.array([0, 1, 1, 0])
    base = torch.tensor(rng.random(SHAPE) * 0.3, device='cuda', requires_grad=True)
    ln = torch.tensor(lines, device='cuda', requires_grad=True)
    img = autograd.draw_lines_fn(ln, torch.tensor(idxs, device='cuda'), out0=base,
                                 max_val=1.0, kernel='biweight', overlap='max')
    g = torch.tensor(rng.random(SHAPE), device='cuda')
    (img * g).sum().backward()
    winner = torch.empty(SHAPE, dtype=torch.int32, device='cuda')
    autograd.lines_backward(g, ln.detach(), torch.tensor(idxs, device='cuda'), 1.0,
                            'biweight', 'max', image=img.detach(), out0=base.detach(),
                            winner=winner)
    w = winner.cpu().numpy()
    assert np.all((w == _native.NO_WINNER) | ((w >= 0) & (w < len(lines))))
    assert (w >= 0).any()
    free = torch.tensor(w == _native.NO_WINNER, device='cuda')
    assert torch.equal(base.grad, torch.where(free, g, torch.zeros_like(g)))
    assert torch.all(ln.grad.abs().sum(1) > 0)


def test_gradient3d_index_forms_and_errors(cuda):
    """int32 and int64 frame indices give the same gradient; no indices draws line i
    into volume i; an index beyond the volumes raises IndexError as the forward does"""
    rng = np.random.default_rng(55)
    lines = random_lines(rng, 5)
    g = torch.tensor(rng.random(SHAPE), device='cuda')
    ln = torch.tensor(lines, device='cuda')
    i32 = torch.tensor(rng.integers(0, SHAPE[0], 5), dtype=torch.int32, device='cuda')
    for overlap in ('sum', 'max'):
        img = torch.zeros(SHAPE, dtype=torch.float64, device='cuda')
        draw_lines(img, ln, i32, 1.2, 'biweight', overlap)
        image = img if overlap == 'max' else None
        a = autograd.lines_backward(g, ln, i32, 1.2, 'biweight', overlap, image=image)
        b = autograd.lines_backward(g, ln, i32.long(), 1.2, 'biweight', overlap, image=image)
        # the per-line sums are double atomics, added in any order
        torch.testing.assert_close(a, b, rtol=1e-12, atol=1e-12)
        assert bool(a.abs().sum() > 0)
    per_line = (5,) + SHAPE[1:]
    g5 = torch.tensor(rng.random(per_line), device='cuda')
    img = torch.zeros(per_line, dtype=torch.float64, device='cuda')
    draw_lines(img, ln, None, 1.2, 'biweight', 'sum')
    none = autograd.lines_backward(g5, ln, None, 1.2, 'biweight', 'sum')
    each = autograd.lines_backward(g5, ln, torch.arange(5, device='cuda'), 1.2, 'biweight', 'sum')
    torch.testing.assert_close(none, each, rtol=1e-12, atol=1e-12)
    bad = i32.clone()
    bad[2] = SHAPE[0]
    with pytest.raises(IndexError):
        autograd.lines_backward(g, ln, bad, 1.2, 'biweight', 'sum')
