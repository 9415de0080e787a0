"""Streak containers that feed the rasteriser: the reference's line containers and
their draw_lines caller (cbclib_v2/_src/streaks.py:10-131), on torch tensors (CUDA or
CPU) or NumPy arrays, plus a fit of the streaks to a measured pattern (fit.fit_lines).

``Lines`` holds (..., 2 * ndim) rows [x0, y0, x1, y1] (2-D) or [x0, y0, z0, x1, y1, z1]
(3-D); ``Streaks`` adds the frame index of every streak, ``StackedStreaks`` a module
index as well.  ``to_lines(width)`` appends
the width column the rasteriser takes, and ``Streaks.pattern_image`` draws the streaks
into frames with ``draw_lines`` (sum overlap, max_val 1), as the reference's
``BaseStreaks.pattern_image`` does (streaks.py:110-131).
"""
from dataclasses import dataclass
from typing import Optional, Sequence, Union

import numpy as np
import torch

from . import fit as _fit
from . import ndimage

Array = Union[torch.Tensor, np.ndarray]


def _is_torch(a) -> bool:
    return isinstance(a, torch.Tensor)


def _sum(a: Array, axis: int) -> Array:
    return a.sum(dim=axis) if _is_torch(a) else a.sum(axis=axis)


def _sqrt(a: Array) -> Array:
    return torch.sqrt(a) if _is_torch(a) else np.sqrt(a)


def _clip(a: Array, lo: float, hi: float) -> Array:
    return a.clamp(lo, hi) if _is_torch(a) else np.clip(a, lo, hi)


class _LineGeometry:
    """The geometry of the segments in ``self.lines`` (reference: BaseLines,
    streaks.py:10-78)."""
    lines: Array

    @property
    def ndim(self) -> int:
        return self.lines.shape[-1] // 2

    @property
    def pt0(self) -> Array:
        return self.lines[..., :self.ndim]

    @property
    def pt1(self) -> Array:
        return self.lines[..., self.ndim:]

    @property
    def points(self) -> Array:
        return self.lines.reshape(tuple(self.lines.shape[:-1]) + (2, self.ndim))

    @property
    def x(self) -> Array:
        return self.lines[..., ::self.ndim]

    @property
    def y(self) -> Array:
        return self.lines[..., 1::self.ndim]

    @property
    def length(self) -> Array:
        return _sqrt(_sum((self.pt1 - self.pt0) ** 2, -1))

    def intersection(self, other: 'Lines') -> Array:
        """Where the (infinite) 2-D lines through self and other cross
        (streaks.py:40-47)."""
        def cross(a, b):
            return a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]

        tau = self.pt1 - self.pt0
        other_tau = other.pt1 - other.pt0
        t = cross(other.pt0 - self.pt0, other_tau) / cross(tau, other_tau)
        return self.pt0 + t[..., None] * tau

    def project(self, point: Array) -> Array:
        """The point of each segment nearest to ``point`` (streaks.py:49-55)."""
        tau = self.pt1 - self.pt0
        center = 0.5 * (self.pt0 + self.pt1)
        r_tau = _sum(tau * (point - center), -1) / _sum(tau ** 2, -1)
        return tau * _clip(r_tau[..., None], -0.5, 0.5) + center

    def distance(self, point: Array) -> Array:
        """Distance from ``point`` to each segment (streaks.py:57-59)."""
        return _sqrt(_sum((self.project(point) - point) ** 2, -1))

    def to_lines(self, width: Union[float, Sequence[float], Array, None] = None) -> Array:
        """The rasteriser's line rows: the segments with a width column appended
        (broadcast from ``width``), or the rows as they are when width is None
        (streaks.py:61-78)."""
        if width is None:
            return self.lines
        shape = tuple(self.lines.shape[:-1]) + (1,)
        if _is_torch(self.lines):
            w = torch.as_tensor(width, dtype=self.lines.dtype, device=self.lines.device)
        else:
            w = np.asarray(width, dtype=self.lines.dtype)
        if tuple(w.shape) == shape[:-1] and w.ndim:
            w = w[..., None]              # one width per line (the reference takes (..., 1))
        if _is_torch(self.lines):
            return torch.cat((self.lines, torch.broadcast_to(w, shape)), dim=-1)
        return np.concatenate((self.lines, np.broadcast_to(w, shape)), axis=-1)


@dataclass
class Lines(_LineGeometry):
    """Line segments (reference: Lines, streaks.py:82-84)."""
    lines: Array


class _StreakMethods(_LineGeometry):
    """Streaks: segments with the frame each belongs to, ``flat_index`` (reference:
    BaseStreaks, streaks.py:86-131)."""

    def _check(self):
        if tuple(self.flat_index.shape) != tuple(self.lines.shape[:-1]):
            raise ValueError(f"index shape {tuple(self.flat_index.shape)} does not match "
                             f"the lines {tuple(self.lines.shape[:-1])}")

    @staticmethod
    def _xy_lines(x: Array, y: Array) -> Array:
        if _is_torch(x):
            return torch.stack((x[..., 0], y[..., 0], x[..., 1], y[..., 1]), dim=-1)
        return np.stack((x[..., 0], y[..., 0], x[..., 1], y[..., 1]), axis=-1)

    def pattern_image(self, out: Array, width: float, kernel: str = 'gaussian') -> Array:
        """Draw the streaks into ``out`` (frames indexed by ``index``) with
        draw_lines: sum overlap, max_val 1 (streaks.py:107-128).  Returns out."""
        return ndimage.draw_lines(out, self.to_lines(width), self.flat_index, kernel=kernel)

    def fit(self, target: torch.Tensor, width: Union[float, Array], kernel: str = 'gaussian',
            overlap: str = 'sum', max_val: float = 1.0, steps: int = 100, lr: float = 0.05,
            min_width: float = 0.5) -> 'FittedStreaks':
        """Refine the streaks' end points and widths so that their pattern matches
        ``target`` (CUDA frames): Adam on sum((pattern - target)^2) through the fused
        render / loss / adjoint steps of fit.fit_lines (2-D streaks)."""
        if self.ndim != 2:
            raise ValueError("fit takes 2-D streaks")
        lines0 = self.to_lines(width)
        lines0 = torch.as_tensor(lines0, dtype=target.dtype, device=target.device)
        idxs = torch.as_tensor(self.flat_index, device=target.device)
        res = _fit.fit_lines(target, lines0, idxs, max_val=max_val, kernel=kernel,
                             overlap=overlap, steps=steps, lr=lr, min_width=min_width)
        d = 2 * self.ndim
        return FittedStreaks(Streaks(index=idxs, lines=res.lines[:, :d].detach()),
                             res.lines[:, d].detach(), res)


@dataclass
class Streaks(_StreakMethods):
    """Streaks in frames ``index`` (reference: Streaks, streaks.py:143-168)."""
    index: Array
    lines: Array

    def __post_init__(self):
        self._check()

    @property
    def flat_index(self) -> Array:
        return self.index

    @classmethod
    def import_xy(cls, index: Array, x: Array, y: Array) -> 'Streaks':
        """Streaks from (..., 2) end-point coordinates (streaks.py:100-105, 153-156)."""
        return cls(index=index, lines=cls._xy_lines(x, y))

    def concentric_only(self, x_ctr: float, y_ctr: float, threshold: float = 0.33) -> Array:
        """The streaks that point at (x_ctr, y_ctr): the part of the centre's offset
        across the streak's normal, relative to the offset, below ``threshold``
        (streaks.py:158-167)."""
        ln = self.lines
        centers = 0.5 * (ln[:, 0:2] + ln[:, 2:4])
        if _is_torch(ln):
            norm = torch.stack([ln[:, 3] - ln[:, 1], ln[:, 0] - ln[:, 2]], dim=-1)
            r = centers - torch.as_tensor([x_ctr, y_ctr], dtype=ln.dtype, device=ln.device)
        else:
            norm = np.stack([ln[:, 3] - ln[:, 1], ln[:, 0] - ln[:, 2]], axis=-1)
            r = centers - np.asarray([x_ctr, y_ctr], dtype=ln.dtype)
        prod = _sum(norm * r, -1)[..., None]
        proj = r - prod * norm / _sum(norm ** 2, -1)[..., None]
        return _sqrt(_sum(proj ** 2, -1)) / _sqrt(_sum(r ** 2, -1)) < threshold


@dataclass
class StackedStreaks(_StreakMethods):
    """Streaks of a detector of ``num_modules`` modules: frame num_modules * index +
    module_id (reference: StackedStreaks, streaks.py:170-190)."""
    index: Array
    module_id: Array
    lines: Array
    num_modules: int = 1

    def __post_init__(self):
        self._check()

    @property
    def flat_index(self) -> Array:
        return self.num_modules * self.index + self.module_id

    @classmethod
    def import_xy(cls, index: Array, module_id: Array, x: Array, y: Array,
                  num_modules: int = 1) -> 'StackedStreaks':
        return cls(index=index, module_id=module_id, lines=cls._xy_lines(x, y),
                   num_modules=num_modules)


@dataclass
class FittedStreaks:
    """The result of Streaks.fit: the refined streaks, their widths and the fit's
    record (losses per step)."""
    streaks: Streaks
    width: torch.Tensor
    result: '_fit.FitResult'
