"""This library against the reference project's own GPU module (cuda_draw_lines,
built unmodified for sm_103a from sources staged into oracle/_ref/cuda_src; skipped
where they are absent).

The reference's GPU path is not its CPU path: it evaluates each pixel's distance in
closed form (cuda_draw_lines.cu:31-42) where the CPU walk accumulates the error
incrementally (bresenham.hpp:38-80, 279-296).  This library follows the CPU path bit
for bit (pinned by the oracle), so against the GPU module:
* rectangular / max, where a pixel is max_val or untouched, the two agree except at
  pixels that lie on a line's support edge (distance = width to within 1e-4 of the
  width, the spread of the two float32 evaluations), checked here in float64 for
  every differing pixel;
* a zero-length segment draws a disc of radius `width` on the reference GPU path
  and nothing on its CPU path (and here), as the reference's own two paths differ.
"""
import numpy as np
import pytest
import torch

from cbclib_v2_gb300 import draw_lines, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def ref_module(cuda):
    from oracle import ref_cuda
    if not ref_cuda.staged() and ref_cuda.module(build_if_missing=False) is None:
        pytest.skip("reference CUDA sources not staged (oracle/build_ref_cuda.sh stage)")
    return ref_cuda.module()


def segment_distance(px, py, lines):
    """float64 distance of pixel (px, py) to each segment (x0, y0, x1, y1)"""
    p0 = lines[:, 0:2]
    t = lines[:, 2:4] - p0
    mag = (t ** 2).sum(1)
    s = np.clip(((px - p0[:, 0]) * t[:, 0] + (py - p0[:, 1]) * t[:, 1]) / np.where(mag > 0, mag, 1),
                0.0, 1.0)
    return np.hypot(p0[:, 0] + s * t[:, 0] - px, p0[:, 1] + s * t[:, 1] - py)


def test_rectangular_max_agrees_except_support_edge_ties(ref_module):
    ls = workloads.detector_stack(seed=77, F=4, H=700, W=650, mean_lines=1500)
    lines = torch.from_numpy(ls.lines.astype(np.float32)).cuda()
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).cuda()
    ref = torch.zeros(ls.shape, device='cuda')
    ref_module.draw_lines(ref, lines, idxs, 1.0, 'rectangular', 'max')
    ours = torch.zeros(ls.shape, device='cuda')
    draw_lines(ours, lines, idxs, 1.0, 'rectangular', 'max')
    torch.cuda.synchronize()
    diff = (ref != ours).nonzero().cpu().numpy()
    drawn = int((ours != 0).sum())
    assert drawn > 0 and len(diff) <= 1e-4 * drawn, (len(diff), drawn)
    l32 = ls.lines.astype(np.float32).astype(np.float64)
    worst = 0.0
    for f, y, x in diff:
        mine = l32[ls.idxs == f]
        d = segment_distance(float(x), float(y), mine)
        worst = max(worst, float(np.abs(d / mine[:, 4] - 1.0).min()))
    # both paths round d / w in float32, the CPU walk through an error accumulated
    # over the walk (float32 increments), so ties spread over ~1e-5 of the width
    print(f"{len(diff)} of {drawn} drawn pixels differ; farthest from a support edge: "
          f"{worst:.2e} of the width")
    assert worst < 1e-4, worst


def test_zero_length_segment_paths_differ(ref_module):
    line = torch.tensor([[20.0, 15.0, 20.0, 15.0, 3.0]], device='cuda')
    ref = torch.zeros((1, 40, 40), device='cuda')
    ref_module.draw_lines(ref, line, torch.zeros(1, dtype=torch.int32, device='cuda'), 1.0,
                          'rectangular', 'max')
    ours = torch.zeros((1, 40, 40), device='cuda')
    draw_lines(ours, line, None, 1.0, 'rectangular', 'max')
    assert int((ref > 0).sum()) > 0                  # a disc on the reference GPU path
    assert int((ours != 0).sum()) == 0               # nothing, as on its CPU path
