"""Seeded synthetic line sets with the shapes and distributions of the benchmark
workloads (no dataset ships with the reference; these stand in for detector frames).

Every generator returns float64 NumPy arrays ``lines`` (N, 5) = [x0, y0, x1, y1, w]
and ``idxs`` (N,) frame indices sorted by frame, plus the frame shape.
"""
from dataclasses import dataclass
from typing import Tuple

import numpy as np


@dataclass
class LineSet:
    name: str
    shape: Tuple[int, int, int]      # (frames, height, width)
    lines: np.ndarray                # (N, 5) float64
    idxs: np.ndarray                 # (N,) int64, non-decreasing
    kernel: str
    overlap: str
    max_val: float = 1.0

    @property
    def n_lines(self) -> int:
        return int(self.lines.shape[0])

    def frame_offsets(self) -> np.ndarray:
        """CSR offsets (F + 1,) of the lines of each frame."""
        return np.searchsorted(self.idxs, np.arange(self.shape[0] + 1)).astype(np.int64)


def _segments(rng, n, H, W, lengths, widths):
    p0 = rng.random((n, 2)) * np.array([W, H], dtype=np.float64)
    ang = rng.random(n) * 2.0 * np.pi
    p1 = p0 + lengths[:, None] * np.stack([np.cos(ang), np.sin(ang)], axis=-1)
    return np.concatenate([p0, p1, widths[:, None]], axis=-1)


def single_frame(seed: int = 0, H: int = 512, W: int = 512, n: int = 1000) -> LineSet:
    """One 512x512 frame, 1,000 segments: uniform endpoints, length U(10, 100),
    width U(1, 5), rectangular profile, sum overlap."""
    rng = np.random.default_rng(seed)
    lines = _segments(rng, n, H, W, rng.uniform(10, 100, n), rng.uniform(1, 5, n))
    return LineSet('single_frame_512', (1, H, W), lines, np.zeros(n, np.int64),
                   'rectangular', 'sum')


def detector_stack(seed: int = 0, F: int = 64, H: int = 2167, W: int = 2070,
                   mean_lines: float = 2000.0) -> LineSet:
    """64 detector frames of 2167x2070: Poisson(2,000) segments per frame, uniform
    endpoints, lognormal length (median 40 px, sigma 0.6) clipped to [5, 400],
    width U(1.5, 4), gaussian profile, max overlap."""
    rng = np.random.default_rng(seed)
    counts = rng.poisson(mean_lines, F)
    n = int(counts.sum())
    lengths = np.clip(rng.lognormal(np.log(40.0), 0.6, n), 5.0, 400.0)
    lines = _segments(rng, n, H, W, lengths, rng.uniform(1.5, 4.0, n))
    idxs = np.repeat(np.arange(F, dtype=np.int64), counts)
    return LineSet(f'detector_stack_{F}x{H}x{W}', (F, H, W), lines, idxs, 'gaussian', 'max')


def ragged_stack(seed: int = 0, F: int = 256, H: int = 1024, W: int = 1024,
                 median: float = 1500.0, sigma: float = 1.0) -> LineSet:
    """256 frames of 1024x1024 with lognormal segment counts (median 1,500, sigma 1.0)
    clipped to [100, 20,000]; segments as in the single-frame workload; triangular
    profile, sum overlap."""
    rng = np.random.default_rng(seed)
    counts = np.clip(np.round(rng.lognormal(np.log(median), sigma, F)), 100, 20000).astype(int)
    n = int(counts.sum())
    lines = _segments(rng, n, H, W, rng.uniform(10, 100, n), rng.uniform(1, 5, n))
    idxs = np.repeat(np.arange(F, dtype=np.int64), counts)
    return LineSet(f'ragged_stack_{F}x{H}x{W}', (F, H, W), lines, idxs, 'triangular', 'sum')


def frames_subset(ls: LineSet, frames) -> LineSet:
    """The lines of some frames, re-indexed 0..len(frames)-1 (for CPU checks)."""
    frames = np.asarray(frames, dtype=np.int64)
    sel = np.isin(ls.idxs, frames)
    remap = {int(f): i for i, f in enumerate(frames)}
    idxs = np.array([remap[int(f)] for f in ls.idxs[sel]], dtype=np.int64)
    return LineSet(ls.name + '_subset', (len(frames), ls.shape[1], ls.shape[2]),
                   ls.lines[sel], idxs, ls.kernel, ls.overlap, ls.max_val)


def fit_stack(seed: int = 0, F: int = 8, H: int = 1024, W: int = 1024,
              per_frame: int = 5000) -> LineSet:
    """8 frames of 1024x1024 with 5,000 segments each, distributed as in the
    single-frame workload; biweight profile (C1, so gradients are meaningful), sum
    overlap.  max_val puts a single line's peak at 100 counts."""
    rng = np.random.default_rng(seed)
    n = F * per_frame
    lines = _segments(rng, n, H, W, rng.uniform(10, 100, n), rng.uniform(1, 5, n))
    idxs = np.repeat(np.arange(F, dtype=np.int64), per_frame)
    return LineSet(f'fit_stack_{F}x{H}x{W}', (F, H, W), lines, idxs, 'biweight', 'sum',
                   max_val=100.0 / 0.9375)


def fit_loop_stack(seed: int = 0, F: int = 32, H: int = 2167, W: int = 2070,
                   per_frame: int = 5000) -> LineSet:
    """32 detector frames of 2167x2070 with 5,000 segments each, distributed as in the
    single-frame workload; biweight profile, max overlap, a single line's peak at 100
    counts.  The streak-fit loop starts from these lines perturbed by N(0, 1 px) on
    the endpoints and N(0, 0.3 px) on the widths."""
    rng = np.random.default_rng(seed)
    n = F * per_frame
    lines = _segments(rng, n, H, W, rng.uniform(10, 100, n), rng.uniform(1, 5, n))
    idxs = np.repeat(np.arange(F, dtype=np.int64), per_frame)
    return LineSet(f'fit_loop_stack_{F}x{H}x{W}', (F, H, W), lines, idxs, 'biweight', 'max',
                   max_val=100.0 / 0.9375)


def perturbed(lines: np.ndarray, seed: int, sigma_pt: float = 0.5,
              sigma_w: float = 0.2) -> np.ndarray:
    """lines with endpoints moved by N(0, sigma_pt) and widths by N(0, sigma_w)"""
    rng = np.random.default_rng(seed)
    out = lines.copy()
    out[:, :4] += rng.normal(0.0, sigma_pt, (lines.shape[0], 4))
    out[:, 4] = np.maximum(out[:, 4] + rng.normal(0.0, sigma_w, lines.shape[0]), 0.5)
    return out


@dataclass
class TermSet:
    """accumulate_lines inputs: line i belongs to term terms[i], term t to frame
    frames[t]; lines are (N, 5) for frames or (N, 7) for volumes"""
    name: str
    shape: Tuple[int, ...]           # (frames, height, width) or (frames, depth, height, width)
    lines: np.ndarray
    terms: np.ndarray                # (N,) int64
    frames: np.ndarray               # (T,) int64
    kernel: str
    in_overlap: str
    out_overlap: str
    max_val: float = 1.0

    @property
    def n_lines(self) -> int:
        return int(self.lines.shape[0])

    def subset(self, n_frames: int) -> 'TermSet':
        """the terms (and their lines) of the first n_frames frames"""
        keep_t = np.flatnonzero(self.frames < n_frames)
        remap = -np.ones(self.frames.size, np.int64)
        remap[keep_t] = np.arange(keep_t.size)
        keep_l = np.flatnonzero(np.isin(self.terms, keep_t))
        return TermSet(self.name, (n_frames,) + tuple(self.shape[1:]), self.lines[keep_l],
                       remap[self.terms[keep_l]], self.frames[keep_t], self.kernel,
                       self.in_overlap, self.out_overlap, self.max_val)


def rotomap_stack(seed: int = 0, F: int = 4, D: int = 96, streaks: int = 500,
                  per_streak: int = 8) -> TermSet:
    """accumulate_lines as the indexer's rotomap calls it: F rotation-space volumes of
    D^3 voxels; each volume has `streaks` terms (streaks) of `per_streak` 3-D
    segments (candidate tilt lines: uniform start, isotropic direction, length
    U(10, 60) voxels, width 2), combined with max within a streak and summed over the
    streaks; gaussian profile."""
    rng = np.random.default_rng(seed)
    n_terms = F * streaks
    n = n_terms * per_streak
    p0 = rng.random((n, 3)) * D
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    p1 = p0 + v * rng.uniform(10, 60, n)[:, None]
    lines = np.concatenate([p0, p1, np.full((n, 1), 2.0)], axis=1)
    terms = np.repeat(np.arange(n_terms, dtype=np.int64), per_streak)
    frames = np.repeat(np.arange(F, dtype=np.int64), streaks)
    return TermSet(f'rotomap_{F}x{D}^3', (F, D, D, D), lines, terms, frames, 'gaussian',
                   'max', 'sum')


def accumulate_stack(seed: int = 0, F: int = 16, H: int = 1024, W: int = 1024,
                     terms_per_frame: int = 1000, per_term: int = 4) -> TermSet:
    """2-D accumulate_lines with mixed overlaps: F frames of H x W, terms of
    `per_term` segments of the single-frame distribution (length U(10, 100), width
    U(1, 5)) summed within a term, the terms combined with max; triangular profile."""
    rng = np.random.default_rng(seed)
    n_terms = F * terms_per_frame
    n = n_terms * per_term
    lines = _segments(rng, n, H, W, rng.uniform(10, 100, n), rng.uniform(1, 5, n))
    terms = np.repeat(np.arange(n_terms, dtype=np.int64), per_term)
    frames = np.repeat(np.arange(F, dtype=np.int64), terms_per_frame)
    return TermSet(f'accumulate_{F}x{H}x{W}', (F, H, W), lines, terms, frames, 'triangular',
                   'sum', 'max')
