"""Generate the golden fixtures of this directory from the reference project's own
compiled CPU module (``bresenham``, built from the reference sources by
oracle/build_ref.sh).  Each fixture stores seeded inputs and the reference's outputs
(single-threaded, so sums are in line order) as compressed .npz.

Run from the repository root:  python tests/golden/make_golden.py
A case without an ``out0`` field starts from zeros of the result's shape and dtype.
Cases follow the reference test-suite (tests/draw_line_test.py:16-112: shapes
(4,3,16,22) / (2,20,16,22), 43 lines, length 10, width 2, max_val 1 and 10) and the
benchmark workloads' line distributions at small sizes, plus edge cases.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

KERNELS = ['biweight', 'gaussian', 'parabolic', 'rectangular', 'triangular']


def reftest_lines(rng, shape, ndim, n_lines=43, length=10.0, width=2.0):
    """tests/draw_line_test.py:95-102 distribution: random start, length 10*U,
    gaussian direction, then Lines.to_lines(width)."""
    lengths = length * rng.random(n_lines)
    pt0 = np.array(shape[:-ndim - 1:-1], dtype=np.float64) * rng.random((n_lines, ndim))
    vec = rng.normal(size=(n_lines, ndim))
    pt1 = pt0 + vec * (lengths / np.sqrt(np.sum(vec**2, axis=-1)))[:, None]
    return np.concatenate([pt0, pt1, np.full((n_lines, 1), width)], axis=-1)


def segment_lines(rng, n, H, W, lmin=10.0, lmax=100.0, wmin=1.0, wmax=5.0):
    """uniform endpoints, uniform lengths and widths, uniform angle"""
    p0 = rng.random((n, 2)) * np.array([W, H])
    ang = rng.random(n) * 2 * np.pi
    ln = rng.uniform(lmin, lmax, n)
    p1 = p0 + ln[:, None] * np.stack([np.cos(ang), np.sin(ang)], axis=-1)
    w = rng.uniform(wmin, wmax, n)
    return np.concatenate([p0, p1, w[:, None]], axis=-1)


def edge_lines(rng, H, W):
    cases = {}
    n = 120
    cases['int_coords'] = np.c_[rng.integers(0, W, (n, 1)), rng.integers(0, H, (n, 1)),
                                rng.integers(0, W, (n, 1)), rng.integers(0, H, (n, 1)),
                                rng.integers(1, 5, (n, 1))].astype(np.float64)
    cases['half_coords'] = np.c_[rng.integers(0, 2 * W, (n, 4)) / 2,
                                 rng.integers(1, 10, (n, 1)) / 2]
    k = np.arange(20, dtype=np.float64)
    cases['diagonal'] = np.c_[k * 3, k + 2, k * 3 + 25, k + 27, np.full(20, 2.0)]
    cases['axis_aligned'] = np.array([[5, 10, 50, 10, 2], [10, 5, 10, 50, 3],
                                      [3.5, 7.5, 40.5, 7.5, 1.5], [60, 2, 60, 55, 4.2],
                                      [50, 30, 5, 30, 2.5], [20, 55, 20, 3, 1.0]])
    cases['outside'] = np.c_[rng.uniform(-60, W + 60, (n, 1)), rng.uniform(-60, H + 60, (n, 1)),
                             rng.uniform(-60, W + 60, (n, 1)), rng.uniform(-60, H + 60, (n, 1)),
                             rng.uniform(0.5, 6, (n, 1))]
    tiny = np.c_[rng.uniform(0, W, (60, 1)), rng.uniform(0, H, (60, 1)), np.zeros((60, 2)),
                 rng.uniform(0.5, 4, (60, 1))]
    tiny[:, 2:4] = tiny[:, 0:2] + rng.normal(0, 1e-3, (60, 2))
    tiny[:20, 2:4] = tiny[:20, 0:2]
    cases['tiny'] = tiny
    cases['widths'] = np.c_[rng.uniform(0, W, (n, 1)), rng.uniform(0, H, (n, 1)),
                            rng.uniform(0, W, (n, 1)), rng.uniform(0, H, (n, 1)),
                            rng.uniform(-2, 0.7, (n, 1))]
    cases['thick'] = np.c_[rng.uniform(0, W, (30, 1)), rng.uniform(0, H, (30, 1)),
                           rng.uniform(0, W, (30, 1)), rng.uniform(0, H, (30, 1)),
                           rng.uniform(5, 25, (30, 1))]
    return cases


def main():
    ref = oracle.reference_module()
    if ref is None:
        raise SystemExit("reference module missing: run oracle/build_ref.sh first")
    rng = np.random.default_rng(20261203)
    out = {}

    # the reference test-suite's own setup (float64, idxs = frames[terms])
    for ndim, shape in ((2, (4, 3, 16, 22)), (3, (2, 20, 16, 22))):
        nfr = int(np.prod(shape[:-ndim]))
        lines = reftest_lines(rng, shape, ndim)
        terms = rng.integers(0, 9, size=43)
        frames = rng.integers(0, nfr - 1, size=10)
        idxs = frames[terms]
        for dtype in ((np.float64, np.float32) if ndim == 2 else (np.float64,)):
            for kernel in KERNELS:
                for max_val in ((1.0, 10.0) if ndim == 2 else (10.0,)):
                    for overlap in ('sum', 'max'):
                        o = np.zeros(shape, dtype)
                        it = np.int64 if dtype == np.float64 else np.int32
                        ref.draw_lines(o, lines.astype(dtype), idxs.astype(it), max_val, kernel,
                                       overlap, 1)
                        key = f"reftest{ndim}d_{np.dtype(dtype).name}_{kernel}_{max_val:g}_{overlap}"
                        out[key] = dict(kind='draw', ndim=ndim, shape=np.array(shape),
                                        lines=lines.astype(dtype), idxs=idxs, max_val=max_val,
                                        kernel=kernel, overlap=overlap, result=o)
                acc = np.zeros(shape, dtype)
                ref.accumulate_lines(acc, lines.astype(dtype), terms.astype(it),
                                     frames.astype(it), 1.0, kernel, 'max', 'sum', 1)
                out[f"acc{ndim}d_{np.dtype(dtype).name}_{kernel}_max_sum"] = dict(
                    kind='accumulate', ndim=ndim, shape=np.array(shape),
                    lines=lines.astype(dtype), terms=terms, frames=frames, max_val=1.0,
                    kernel=kernel, in_overlap='max', out_overlap='sum', result=acc)

    # single frame, segment distribution of the 512x512 workload at 128x144
    H, W = 128, 144
    lines = segment_lines(rng, 200, H, W).astype(np.float32)
    for kernel in KERNELS:
        for overlap in ('sum', 'max'):
            o0 = np.full((1, H, W), 0.5 if overlap == "sum" else 0.0, np.float32)
            o = o0.copy()
            ref.draw_lines(o, lines, None, 2.5, kernel, overlap, 1)
            out[f"frame_f32_{kernel}_{overlap}"] = dict(
                kind='draw', ndim=2, shape=np.array(o.shape), lines=lines, idxs=None,
                max_val=2.5, kernel=kernel, overlap=overlap, out0=o0, result=o)

    # edge cases on a 60x70 frame
    for name, ln in edge_lines(rng, 60, 70).items():
        for kernel in ('gaussian', 'biweight', 'rectangular'):
            for overlap in ('sum', 'max'):
                o = np.zeros((60, 70), np.float32)
                ref.draw_lines(o, ln.astype(np.float32), None, 3.0, kernel, overlap, 1)
                out[f"edge_{name}_{kernel}_{overlap}"] = dict(
                    kind='draw', ndim=2, shape=np.array(o.shape), lines=ln.astype(np.float32),
                    idxs=None, max_val=3.0, kernel=kernel, overlap=overlap, result=o)

    flat = {}
    for key, case in out.items():
        for field, val in case.items():
            if val is None:
                continue
            flat[f"{key}/{field}"] = np.asarray(val)
    path = os.path.join(HERE, 'draw_lines_golden.npz')
    np.savez_compressed(path, **flat)
    print(f"wrote {len(out)} cases to {path} ({os.path.getsize(path) / 1e3:.0f} kB)")


if __name__ == '__main__':
    main()
