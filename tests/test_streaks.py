"""Streak containers (the reference's Lines / Streaks / StackedStreaks, which feed
draw_lines through Streaks.pattern_image, cbclib_v2/_src/streaks.py:10-190): geometry on
the CPU against direct formulas, pattern_image against the oracle's draw_lines and the
streak fit on the GPU."""
import numpy as np
import pytest
import torch

import oracle
from cbclib_v2_gb300 import Lines, StackedStreaks, Streaks


def _streaks(seed=0, n=40, F=3, H=60, W=80):
    rng = np.random.default_rng(seed)
    p0 = rng.random((n, 2)) * [W, H]
    p1 = p0 + rng.normal(scale=15, size=(n, 2))
    return Streaks(index=rng.integers(0, F, n), lines=np.concatenate([p0, p1], axis=1))


def test_geometry_numpy_and_torch():
    s = _streaks()
    pt = np.array([30.0, 20.0])
    tau = s.pt1 - s.pt0
    c = 0.5 * (s.pt0 + s.pt1)
    t = np.clip(((pt - c) * tau).sum(-1) / (tau ** 2).sum(-1), -0.5, 0.5)
    proj = c + t[:, None] * tau
    np.testing.assert_allclose(s.length, np.linalg.norm(tau, axis=1))
    np.testing.assert_allclose(s.project(pt), proj)
    np.testing.assert_allclose(s.distance(pt), np.linalg.norm(proj - pt, axis=1))
    assert s.points.shape == (40, 2, 2) and s.ndim == 2
    np.testing.assert_array_equal(s.x, s.lines[:, [0, 2]])
    np.testing.assert_array_equal(s.y, s.lines[:, [1, 3]])
    ts = Streaks(index=torch.from_numpy(s.index), lines=torch.from_numpy(s.lines))
    np.testing.assert_allclose(ts.distance(torch.from_numpy(pt)).numpy(), s.distance(pt))
    a = Lines(np.array([[0.0, 0.0, 2.0, 2.0]]))
    b = Lines(np.array([[0.0, 2.0, 2.0, 0.0]]))
    np.testing.assert_allclose(a.intersection(b), [[1.0, 1.0]])


def test_to_lines_and_indices():
    s = _streaks(1, n=5)
    assert s.to_lines() is s.lines
    ln = s.to_lines(2.5)
    assert ln.shape == (5, 5) and np.all(ln[:, 4] == 2.5)
    np.testing.assert_array_equal(s.to_lines(np.arange(5.0))[:, 4], np.arange(5.0))
    t = Streaks(index=torch.arange(5), lines=torch.from_numpy(s.lines))
    assert torch.equal(t.to_lines(1.5)[:, 4], torch.full((5,), 1.5, dtype=torch.float64))
    st = StackedStreaks(index=np.array([0, 0, 1, 1, 2]), module_id=np.array([0, 1, 0, 1, 0]),
                        lines=s.lines, num_modules=2)
    np.testing.assert_array_equal(st.flat_index, [0, 1, 2, 3, 4])
    xy = Streaks.import_xy(np.arange(5), s.x, s.y)
    np.testing.assert_array_equal(xy.lines, s.lines)
    with pytest.raises(ValueError, match="does not match"):
        Streaks(index=np.arange(4), lines=s.lines)


def test_concentric_only():
    # concentric = along a circle about the centre (the offset of the streak's centre
    # mostly across the streak): two radial streaks from (50, 50), one tangential
    lines = np.array([[60.0, 50.0, 70.0, 50.0], [50.0, 30.0, 50.0, 20.0],
                      [60.0, 40.0, 60.0, 60.0]])
    s = Streaks(index=np.zeros(3, np.int64), lines=lines)
    np.testing.assert_array_equal(s.concentric_only(50.0, 50.0), [False, False, True])


@pytest.mark.gpu
def test_pattern_image_matches_oracle(cuda):
    s = _streaks(2, n=60)
    out = torch.zeros((3, 60, 80), dtype=torch.float32, device='cuda')
    res = s.pattern_image(out, 2.0, kernel='gaussian')
    assert res is out
    ref = oracle.draw_lines(np.zeros((3, 60, 80), np.float32),
                            s.to_lines(2.0).astype(np.float32), s.index, 1.0, 'gaussian', 'sum')
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-5, atol=1e-7)
    # host frames through the device module, as the reference's NumPy callers pass them
    host = np.zeros((3, 60, 80), np.float32)
    s.pattern_image(host, 2.0, kernel='gaussian')
    np.testing.assert_allclose(host, ref, rtol=1e-5, atol=1e-7)


@pytest.mark.gpu
def test_fit_recovers_streaks(cuda):
    rng = np.random.default_rng(4)
    n, F, H, W = 30, 2, 96, 96
    p0 = rng.random((n, 2)) * 60 + 18
    p1 = p0 + rng.normal(scale=12, size=(n, 2))
    truth = Streaks(index=torch.from_numpy(rng.integers(0, F, n)).cuda(),
                    lines=torch.from_numpy(np.concatenate([p0, p1], 1)).float().cuda())
    target = torch.zeros((F, H, W), device='cuda')
    truth.pattern_image(target, 2.0, kernel='biweight')
    start = Streaks(index=truth.index, lines=truth.lines + 0.6 * torch.randn_like(truth.lines))
    fitted = start.fit(target, 2.0, kernel='biweight', steps=150, lr=0.05)
    err0 = (start.lines - truth.lines).pow(2).mean().sqrt()
    err1 = (fitted.streaks.lines - truth.lines).pow(2).mean().sqrt()
    assert fitted.result.losses[-1] < 0.2 * fitted.result.losses[0]
    assert err1 < 0.5 * err0
    assert fitted.width.shape == (n,)
