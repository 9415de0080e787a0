"""The adjoint (gradient of draw_lines with respect to the line parameters) against
central finite differences of the float64 oracle forward, step 1e-3 px, for the loss
L = sum((I - T)^2) with a fixed target T.

Gate: relative error <= 1e-4 (float64 adjoint) on every parameter whose gradient
exceeds 1% of the largest, and on the whole gradient vector in the 2-norm.  The
biweight profile is C1 across its support edge, so finite differences are accurate;
for max overlap the lines are kept apart so that no pixel switches winner."""
import numpy as np
import pytest
import torch

import oracle
from cbclib_v2_gb300 import autograd, draw_lines

pytestmark = pytest.mark.gpu

STEP = 1e-3
RTOL = 1e-4


def separated_lines(rng, nx, ny, cell=40.0):
    """one line per grid cell, short enough to stay inside it"""
    rows = []
    for i in range(nx):
        for j in range(ny):
            c = np.array([cell * (i + 0.5), cell * (j + 0.5)])
            ang = rng.random() * np.pi
            half = rng.uniform(4, 11)
            d = half * np.array([np.cos(ang), np.sin(ang)])
            rows.append([*(c - d), *(c + d), rng.uniform(1.6, 3.8)])
    return np.array(rows)


def oracle_loss(lines, idxs, shape, target, kernel, overlap, max_val):
    img = oracle.draw_lines(np.zeros(shape), lines, idxs, max_val, kernel, overlap, 1)
    return float(np.sum((img - target) ** 2))


def fd_gradient(lines, idxs, shape, target, kernel, overlap, max_val):
    g = np.zeros_like(lines)
    for i in range(lines.shape[0]):
        for k in range(5):
            lp, lm = lines.copy(), lines.copy()
            lp[i, k] += STEP
            lm[i, k] -= STEP
            g[i, k] = (oracle_loss(lp, idxs, shape, target, kernel, overlap, max_val) -
                       oracle_loss(lm, idxs, shape, target, kernel, overlap, max_val)) / (2 * STEP)
    return g


def adjoint_gradient(lines, idxs, shape, target, kernel, overlap, max_val, dtype):
    ln = torch.tensor(lines, dtype=dtype, device='cuda', requires_grad=True)
    ix = torch.tensor(idxs, device='cuda')
    img = autograd.draw_lines_fn(ln, ix, shape=shape, max_val=max_val, kernel=kernel,
                                 overlap=overlap)
    loss = ((img - torch.tensor(target, dtype=dtype, device='cuda')) ** 2).sum()
    loss.backward()
    return ln.grad.double().cpu().numpy(), img.detach().double().cpu().numpy()


def relative_errors(got, want):
    big = np.abs(want) > 0.01 * np.abs(want).max()
    per = np.abs(got - want)[big] / np.abs(want)[big]
    return per.max(), np.linalg.norm(got - want) / np.linalg.norm(want)


@pytest.mark.parametrize("overlap", ['sum', 'max'])
def test_gradient_matches_fp64_finite_differences(cuda, overlap):
    rng = np.random.default_rng(31 if overlap == 'sum' else 32)
    if overlap == 'sum':
        lines = np.c_[rng.uniform(8, 72, (10, 2)), rng.uniform(8, 72, (10, 2)),
                      rng.uniform(1.6, 3.8, (10, 1))]
        idxs = rng.integers(0, 2, 10)
    else:
        lines = separated_lines(rng, 2, 2)
        idxs = np.array([0, 1, 1, 0])
    shape = (2, 80, 84)
    target = rng.random(shape) * 0.5
    kernel, max_val = 'biweight', 1.3
    want = fd_gradient(lines, idxs, shape, target, kernel, overlap, max_val)
    got, img = adjoint_gradient(lines, idxs, shape, target, kernel, overlap, max_val,
                                torch.float64)
    ref = oracle.draw_lines(np.zeros(shape), lines, idxs, max_val, kernel, overlap, 1)
    assert np.allclose(img, ref, rtol=1e-14, atol=1e-15)
    per, norm = relative_errors(got, want)
    assert per <= RTOL and norm <= RTOL, (per, norm)
    got32, _ = adjoint_gradient(lines, idxs, shape, target, kernel, overlap, max_val,
                                torch.float32)
    per32, norm32 = relative_errors(got32, want)
    print(f"float32 adjoint, {overlap}: per parameter {per32:.3e}, 2-norm {norm32:.3e}")
    assert norm32 <= RTOL, (per32, norm32)


def torch_profile(kernel, x):
    if kernel == 'biweight':
        return 0.9375 * (1 - x * x) ** 2
    if kernel == 'gaussian':
        return torch.exp(-(3 * x) ** 2 / 2) / np.sqrt(2 * np.pi)
    if kernel == 'parabolic':
        return 0.75 * (1 - x * x)
    if kernel == 'rectangular':
        return torch.ones_like(x)
    return 1 - x


@pytest.mark.parametrize("overlap", ['sum', 'max'])
@pytest.mark.parametrize("kernel", ['biweight', 'gaussian', 'parabolic', 'rectangular',
                                    'triangular'])
def test_gradient_matches_torch_closed_form(cuda, kernel, overlap):
    """One line per frame: the adjoint equals torch autograd of max_val * K(d / w)
    (d: distance to the segment, tests/draw_line_test.py:154-167 with Lines.project)
    summed over the pixels the forward drew, for every profile (including the
    gaussian, whose jump at the support edge defeats finite differences).  With one
    line per frame every drawn pixel's winner is that line, so max overlap (the pass
    over the pixels' winners) gives the same gradient as sum overlap (the walks)."""
    rng = np.random.default_rng(50)
    lines = separated_lines(rng, 3, 1)
    shape = (3, 40, 40)
    for f in range(3):
        lines[f, [0, 2]] -= 40 * f                # line f in the middle of frame f
    idxs = np.arange(3)
    max_val = 1.7
    target = torch.tensor(rng.random(shape) * 0.3, device='cuda')
    got, img = adjoint_gradient(lines, idxs, shape, target.cpu().numpy(), kernel, overlap,
                                max_val, torch.float64)
    if kernel == 'rectangular':
        assert np.all(got == 0)
        return
    drawn = torch.tensor(img != 0, device='cuda')
    ln = torch.tensor(lines, device='cuda', requires_grad=True)
    yy, xx = torch.meshgrid(torch.arange(40.0, device='cuda', dtype=torch.float64),
                            torch.arange(40.0, device='cuda', dtype=torch.float64), indexing='ij')
    loss = 0
    for f in range(3):
        p0, p1, w = ln[f, :2], ln[f, 2:4], ln[f, 4]
        tau = p1 - p0
        ctr = 0.5 * (p0 + p1)
        t = (((xx - ctr[0]) * tau[0] + (yy - ctr[1]) * tau[1]) / (tau ** 2).sum()).clamp(-0.5, 0.5)
        d2 = (ctr[0] + t * tau[0] - xx) ** 2 + (ctr[1] + t * tau[1] - yy) ** 2
        d = torch.sqrt(torch.clamp(d2, min=1e-30))
        v = torch.where(drawn[f], max_val * torch_profile(kernel, d / w), torch.zeros_like(d))
        loss = loss + ((v - target[f]) ** 2).sum()
    loss.backward()
    want = ln.grad.cpu().numpy()
    assert np.isfinite(want).all()
    assert np.allclose(got, want, rtol=1e-9, atol=1e-9 * np.abs(want).max())


def test_gradient_of_out0_and_winner(cuda):
    rng = np.random.default_rng(5)
    lines = torch.tensor(separated_lines(rng, 2, 1), device='cuda', requires_grad=True)
    out0 = torch.full((1, 80, 40), 0.3, device='cuda', dtype=torch.float64, requires_grad=True)
    img = autograd.draw_lines_fn(lines, None, out0=out0, max_val=1.0, kernel='parabolic',
                                 overlap='max')
    g = torch.randn_like(img)
    img.backward(g)
    kept = (img.detach() == out0.detach())
    assert torch.equal(out0.grad[kept], g[kept])
    assert float(out0.grad[~kept].abs().sum()) == 0.0
    # sum: d(out0 + draw)/d(out0) is the identity
    out1 = out0.detach().clone().requires_grad_(True)
    img = autograd.draw_lines_fn(lines, None, out0=out1, max_val=1.0, kernel='parabolic')
    img.backward(g)
    assert torch.equal(out1.grad, g)


def test_forward_matches_in_place_draw_lines(cuda):
    rng = np.random.default_rng(6)
    lines = np.c_[rng.uniform(0, 200, (300, 4)), rng.uniform(1, 4, (300, 1))].astype(np.float32)
    idxs = rng.integers(0, 3, 300)
    for overlap in ('sum', 'max'):
        a = autograd.draw_lines_fn(torch.tensor(lines, device='cuda'), torch.tensor(idxs, device='cuda'),
                                   shape=(3, 200, 210), kernel='gaussian', overlap=overlap)
        b = torch.zeros((3, 200, 210), device='cuda')
        draw_lines(b, lines, idxs, kernel='gaussian', overlap=overlap)
        if overlap == 'max':
            assert torch.equal(a, b)
        else:                      # sum: the order of float additions may differ
            assert torch.allclose(a, b, rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("kernel", ['biweight', 'gaussian', 'triangular', 'rectangular'])
def test_max_winner_forward_matches_draw_and_winner_pass(cuda, kernel):
    """draw_lines_max_winner: the same frames as draw_lines(max) from zero, and the same
    winners as the adjoint's own winner pass"""
    import numpy as np
    import torch
    from cbclib_v2_gb300 import autograd, ndimage
    rng = np.random.default_rng(21)
    F, H, W, n = 2, 90, 110, 150
    p0 = rng.random((n, 2)) * [W, H]
    v = rng.normal(size=(n, 2))
    p1 = p0 + v / np.linalg.norm(v, axis=1, keepdims=True) * rng.uniform(3, 40, n)[:, None]
    lines = torch.from_numpy(np.concatenate([p0, p1, rng.uniform(1, 5, (n, 1))], 1)
                             .astype(np.float32)).cuda()
    idxs = torch.from_numpy(rng.integers(0, F, n).astype(np.int32)).cuda()
    img = torch.full((F, H, W), 7.0, device='cuda')         # overwritten
    win = ndimage.draw_lines_max_winner(img, lines, idxs, 2.0, kernel)
    ref = torch.zeros((F, H, W), device='cuda')
    ndimage.draw_lines(ref, lines, idxs, 2.0, kernel, 'max')
    assert torch.equal(img, ref)
    w2 = torch.empty((F, H, W), dtype=torch.int32, device='cuda')
    autograd.lines_backward(torch.ones_like(ref), lines, idxs, 2.0, kernel, 'max', ref, None, w2)
    assert torch.equal(win, w2)
    again = torch.empty_like(img)                           # the scratch was left zero
    assert torch.equal(ndimage.draw_lines_max_winner(again, lines, idxs, 2.0, kernel), win)
    assert torch.equal(again, ref)
