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


@pytest.mark.parametrize("overlap", ['max', 'sum'])
def test_fused_squared_loss_gradient_matches_autograd(cuda, overlap):
    """the fused loss adjoint forms 2 (I - T) per drawn pixel: the same gradient as
    torch autograd through draw_lines_fn and a torch loss"""
    from cbclib_v2_gb300 import autograd
    ls = workloads.fit_loop_stack(seed=9, F=2, H=200, W=180, per_frame=80)
    lines = torch.from_numpy(ls.lines.astype(np.float32)).cuda()
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).cuda()
    target = torch.rand(ls.shape, device='cuda',
                        generator=torch.Generator(device='cuda').manual_seed(9)) * 50
    p = lines.clone().requires_grad_(True)
    img = autograd.draw_lines_fn(p, idxs, shape=ls.shape, max_val=ls.max_val, kernel=ls.kernel,
                                 overlap=overlap)
    ((img - target) ** 2).sum().backward()
    image = torch.empty_like(target)
    g = fit.squared_loss_step(image, target, lines, idxs, ls.max_val, ls.kernel, overlap)
    if overlap == 'max':
        assert torch.equal(image, img.detach())
    else:                   # sum overlap: addition order differs between two renders
        torch.testing.assert_close(image, img.detach(), rtol=1e-5, atol=1e-4)
    torch.testing.assert_close(g, p.grad, rtol=1e-5, atol=1e-3)
    if overlap == 'max':           # values and winners packed in one word, no frames
        g2 = fit.squared_loss_step(None, target, lines, idxs, ls.max_val, ls.kernel, overlap)
        torch.testing.assert_close(g2, g, rtol=1e-5, atol=1e-3)


def test_fit_fused_and_autograd_paths_agree(cuda):
    ls = workloads.fit_loop_stack(seed=10, F=1, H=160, W=160, per_frame=40)
    truth = torch.from_numpy(ls.lines.astype(np.float32)).cuda()
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).cuda()
    target = torch.zeros(ls.shape, device='cuda')
    draw_lines(target, truth, idxs, ls.max_val, ls.kernel, 'sum')
    start = torch.from_numpy(workloads.perturbed(ls.lines, 11, 1.0, 0.3).astype(np.float32)).cuda()
    a = fit.fit_lines(target, start, idxs, max_val=ls.max_val, kernel=ls.kernel, overlap='sum',
                      steps=20, fused=True)
    b = fit.fit_lines(target, start, idxs, max_val=ls.max_val, kernel=ls.kernel, overlap='sum',
                      steps=20, fused=False)
    torch.testing.assert_close(a.lines, b.lines, rtol=1e-4, atol=1e-3)


@pytest.mark.parametrize("kernel", ['biweight', 'gaussian', 'parabolic', 'rectangular',
                                    'triangular'])
@pytest.mark.parametrize("shape", [(3, 23, 37), (1, 64, 64), (2, 9, 5)])
def test_packed_loss_step_matches_image_path(cuda, kernel, shape):
    """cbc_squared_loss_step_f32 (forward into packed words, one pass over them and the
    target): the gradient of the image + winner path, the loss minus sum(T^2), and the
    packed scratch left zero; frame sizes that are not multiples of the 8-pixel chunk,
    and a target whose address is not 16-byte aligned (element loads)."""
    from cbclib_v2_gb300 import ndimage
    F, H, W = shape
    rng = np.random.default_rng(F * 1000 + H + W)
    n = 12 * F
    lines = np.empty((n, 5))
    lines[:, 0] = rng.uniform(-3, W + 3, n)
    lines[:, 1] = rng.uniform(-3, H + 3, n)
    lines[:, 2] = lines[:, 0] + rng.uniform(-15, 15, n)
    lines[:, 3] = lines[:, 1] + rng.uniform(-15, 15, n)
    lines[:, 4] = rng.uniform(0.7, 4, n)
    lines = torch.tensor(lines, dtype=torch.float32, device='cuda')
    idxs = torch.tensor(np.repeat(np.arange(F), 12), dtype=torch.int32, device='cuda')
    base = torch.rand(F * H * W + 1, device='cuda') * 3
    for target in (base[:-1].view(shape), base[1:].view(shape)):
        image = torch.empty(shape, device='cuda')
        want = fit.squared_loss_step(image, target, lines, idxs, 1.4, kernel, 'max')
        delta = torch.zeros((), dtype=torch.float64, device='cuda')
        got = fit.squared_loss_step(None, target, lines, idxs, 1.4, kernel, 'max',
                                    loss_delta=delta)
        torch.testing.assert_close(got, want, rtol=1e-5, atol=1e-4)
        loss = float(((image.double() - target.double()) ** 2).sum())
        t2 = float((target.double() ** 2).sum())
        assert abs(t2 + float(delta) - loss) <= 1e-6 * loss
        assert int(ndimage._packed_scratch(target.device, F * H * W).count_nonzero()) == 0
    if kernel == 'rectangular':
        assert torch.all(got == 0)


def test_fit_loss_history(cuda):
    """the fused max path records the loss at the start of every step"""
    ls = workloads.fit_loop_stack(seed=12, F=2, H=128, W=120, per_frame=30)
    truth = torch.from_numpy(ls.lines.astype(np.float32)).cuda()
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).cuda()
    target = torch.zeros(ls.shape, device='cuda')
    draw_lines(target, truth, idxs, ls.max_val, ls.kernel, 'max')
    start = torch.from_numpy(workloads.perturbed(ls.lines, 13, 1.0, 0.3).astype(np.float32)).cuda()
    res = fit.fit_lines(target, start, idxs, max_val=ls.max_val, kernel=ls.kernel,
                        overlap='max', steps=30)
    assert res.history is not None and len(res.history) == 30
    assert abs(res.history[0] - res.losses[0]) <= 1e-6 * res.losses[0]
    assert res.history[-1] < 0.5 * res.history[0]


def test_adam_step_matches_torch_adam(cuda):
    """cbc_adam_step_f32 follows torch.optim.Adam (default betas, eps), then clamps the
    widths"""
    rng = np.random.default_rng(14)
    p0 = torch.tensor(rng.normal(0, 3, (300, 5)), dtype=torch.float32, device='cuda')
    p0[:, 4] = p0[:, 4].abs() + 0.6
    a = p0.clone().requires_grad_(True)
    opt = torch.optim.Adam([a], lr=0.05)
    b = p0.clone()
    m, v = torch.zeros_like(b), torch.zeros_like(b)
    for step in range(1, 8):
        g = torch.tensor(rng.normal(0, 10, (300, 5)), dtype=torch.float32, device='cuda')
        a.grad = g.clone()
        opt.step()
        with torch.no_grad():
            a[:, 4].clamp_(min=0.5)
        fit.adam_step(b, g, m, v, step, 0.05, min_width=0.5)
        torch.testing.assert_close(b, a.detach(), rtol=1e-6, atol=1e-6)
    assert float(b[:, 4].min()) >= 0.5


def test_unchecked_steps_fall_back_when_checkpoints_run_out(cuda, monkeypatch):
    """steps after the first read their status only at the end; a step that ran out of
    walk checkpoints makes the whole fit run again with a check after every step"""
    ls = workloads.fit_loop_stack(seed=15, F=2, H=128, W=120, per_frame=30)
    truth = torch.from_numpy(ls.lines.astype(np.float32)).cuda()
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).cuda()
    target = torch.zeros(ls.shape, device='cuda')
    draw_lines(target, truth, idxs, ls.max_val, ls.kernel, 'max')
    start = torch.from_numpy(workloads.perturbed(ls.lines, 16, 1.0, 0.3).astype(np.float32)).cuda()
    kw = dict(max_val=ls.max_val, kernel=ls.kernel, overlap='max', steps=12)
    want = fit.fit_lines(target, start, idxs, _checked=True, **kw)
    first = fit._PackedSteps.first
    runs = []

    def starved(self, lines, delta):
        g = first(self, lines, delta)
        self.ck = 1                        # no room: every later step overflows
        runs.append(1)
        return g

    monkeypatch.setattr(fit._PackedSteps, 'first', starved)
    got = fit.fit_lines(target, start, idxs, **kw)
    assert len(runs) == 1
    torch.testing.assert_close(got.lines, want.lines, rtol=1e-5, atol=1e-5)
    monkeypatch.setattr(fit._PackedSteps, 'first', first)
    again = fit.fit_lines(target, start, idxs, **kw)
    torch.testing.assert_close(again.lines, want.lines, rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("kernel", ['biweight', 'gaussian', 'triangular'])
def test_sum_loss_step_matches_two_calls(cuda, kernel):
    """cbc_squared_loss_step_sum_f32 (forward, then the adjoint over the forward's own
    checkpoints) against draw_lines followed by the separate adjoint, with lines long
    enough for the long-walk list, int64 indices, and the loss it reports"""
    from cbclib_v2_gb300.autograd import squared_loss_backward
    rng = np.random.default_rng(12)
    F, H, W, n = 3, 150, 260, 300
    p0 = rng.random((n, 2)) * [W, H]
    v = rng.normal(size=(n, 2))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    p1 = p0 + v * rng.uniform(2, 240, n)[:, None]          # some walks beyond 96 columns
    lines = torch.from_numpy(np.concatenate([p0, p1, rng.uniform(0.5, 4, (n, 1))], 1)
                             .astype(np.float32)).cuda()
    idxs = torch.from_numpy(rng.integers(0, F, n)).cuda()
    target = torch.rand((F, H, W), device='cuda') * 3
    image = torch.empty_like(target)
    loss = torch.zeros((), dtype=torch.float64, device='cuda')
    g = fit._sum_loss_step(image, target, lines, idxs, 2.0, kernel, loss)
    ref_img = torch.zeros_like(target)
    draw_lines(ref_img, lines, idxs, 2.0, kernel, 'sum')
    ref_g = squared_loss_backward(ref_img, target, lines, idxs, 2.0, kernel, 'sum')
    torch.testing.assert_close(image, ref_img, rtol=1e-5, atol=1e-5)
    torch.testing.assert_close(g, ref_g, rtol=1e-4, atol=1e-3)
    want = ((ref_img.double() - target.double()) ** 2).sum()
    torch.testing.assert_close(loss, want, rtol=1e-9, atol=1e-6)
    # no lines: zero frames, the loss of the empty image
    g0 = fit._sum_loss_step(image, target, lines[:0], idxs[:0], 2.0, kernel, loss)
    assert g0.shape == (0, 5) and not image.any()
    torch.testing.assert_close(loss, (target.double() ** 2).sum(), rtol=1e-9, atol=1e-6)
