"""Least-squares refinement of line parameters against measured frames with Adam,
through the differentiable draw_lines (forward and adjoint kernels).

This is the loop that follows ``Streaks.pattern_image`` in the reference's workflow
(cbclib_v2/_src/streaks.py:65-131): the lines of detected streaks, drawn with a
profile, are moved so that the drawn frames match the measured ones.  The loss is
sum((draw(lines) - target)^2) over all frames; the widths are kept at or above
``min_width`` after every step (a line of width <= 0 draws nothing and gets no
gradient).
"""
import time
from dataclasses import dataclass, field
from typing import List, Optional

import torch

from . import _native, ndimage
from .autograd import draw_lines_fn, squared_loss_backward

__all__ = ['FitResult', 'ShardedFit', 'adam_step', 'fit_lines', 'fit_lines_sharded',
           'reduce_losses', 'shard_problem', 'squared_loss_step']


@dataclass
class FitResult:
    lines: torch.Tensor                  # (N, 5) fitted parameters
    steps: int
    seconds: float                       # wall time of the steps (synchronised)
    losses: List[float] = field(default_factory=list)   # loss before step 0 and after the last
    history: Optional[List[float]] = None   # loss at the start of every step (fused max path)

    @property
    def ms_per_step(self) -> float:
        return 1e3 * self.seconds / max(self.steps, 1)


def _loss(params, idxs, target, max_val, kernel, overlap):
    img = draw_lines_fn(params, idxs, shape=target.shape, max_val=max_val, kernel=kernel,
                        overlap=overlap)
    return ((img - target) ** 2).sum()


def _packed_loss_step(target: torch.Tensor, lines, idxs, max_val: float, kernel: str,
                      loss_delta: Optional[torch.Tensor] = None) -> torch.Tensor:
    """cbc_squared_loss_step_f32: forward into this thread's packed scratch, gradient
    of sum((draw(lines) - target)^2), scratch zeroed again, in one library call.
    ``loss_delta`` (a float64 CUDA scalar, or None) receives the loss minus
    sum(target^2)."""
    k, _ = ndimage._check_names(kernel, 'max')
    if not (target.is_cuda and target.dtype == torch.float32):
        raise TypeError("target must be a float32 CUDA tensor")
    dev = target.device
    F, H, W = ndimage._frames_of(target)
    ln = ndimage._as_device_lines(lines, dev, torch.float32)
    if ln.shape[1] != 5:
        raise ValueError("the fused loss step takes 2-D lines (N, 5)")
    n = ln.shape[0]
    ix = ndimage._as_device_idxs(idxs, n, dev)
    if ix is None and n and F != 1 and F != n:
        raise ValueError(f"idxs has an incompatible size ({n} != {F})")
    tg = target.contiguous()
    grad = torch.empty((n, 5), dtype=torch.float32, device=dev)
    lib = _native.lib()
    loss_ptr = None if loss_delta is None else loss_delta.data_ptr()

    def call(buf, capacity, ck_capacity, tref, stream):
        packed = ndimage._packed_scratch(dev, F * H * W)
        return lib.cbc_squared_loss_step_f32(
            tg.data_ptr(), F, H, W, ln.data_ptr(), n, None if ix is None else ix.data_ptr(),
            0 if ix is None else ix.element_size(), max_val, k, packed.data_ptr(),
            grad.data_ptr(), loss_ptr, buf.data_ptr(), buf.numel(), capacity, ck_capacity,
            stream)

    ndimage._run_with_workspace(call, dev, F, H, W, n, 4, None,
                                size_fn=lib.cbc_squared_loss_step_workspace_size)
    return grad


def _sum_loss_step(image: torch.Tensor, target: torch.Tensor, lines, idxs, max_val: float,
                   kernel: str, loss: Optional[torch.Tensor] = None) -> torch.Tensor:
    """cbc_squared_loss_step_sum_f32: the sum-overlap forward into ``image`` and the
    gradient of sum((image - target)^2), the adjoint walking the forward's own
    checkpoints, in one library call; ``loss`` (a float64 CUDA scalar, or None)
    receives the loss."""
    k, _ = ndimage._check_names(kernel, 'sum')
    dev = target.device
    F, H, W = ndimage._frames_of(target)
    if tuple(image.shape) != tuple(target.shape) or not image.is_contiguous() or \
            image.device != target.device:
        raise ValueError("image must be a contiguous tensor of the target's shape and device")
    ln = ndimage._as_device_lines(lines, dev, torch.float32)
    if ln.shape[1] != 5:
        raise ValueError("the fused loss step takes 2-D lines (N, 5)")
    n = ln.shape[0]
    ix = ndimage._as_device_idxs(idxs, n, dev)
    if ix is None and n and F != 1 and F != n:
        raise ValueError(f"idxs has an incompatible size ({n} != {F})")
    tg = target.contiguous()
    grad = torch.empty((n, 5), dtype=torch.float32, device=dev)
    lib = _native.lib()
    loss_ptr = None if loss is None else loss.data_ptr()

    def call(buf, capacity, ck_capacity, tref, stream):
        return lib.cbc_squared_loss_step_sum_f32(
            tg.data_ptr(), image.data_ptr(), F, H, W, ln.data_ptr(), n,
            None if ix is None else ix.data_ptr(), 0 if ix is None else ix.element_size(),
            max_val, k, grad.data_ptr(), loss_ptr, buf.data_ptr(), buf.numel(), capacity,
            ck_capacity, stream)

    ndimage._run_with_workspace(call, dev, F, H, W, n, 4, None,
                                size_fn=lib.cbc_squared_loss_step_workspace_size)
    return grad


class _PackedSteps:
    """The fused loss steps of one fit: the first step runs through the checking
    path (which sizes the workspace), later steps enqueue the library call and an
    asynchronous copy of its device status, read once after the last step."""

    def __init__(self, target: torch.Tensor, idxs, max_val: float, kernel: str, n: int,
                 steps: int):
        self.k, _ = ndimage._check_names(kernel, 'max')
        self.dev = target.device
        self.F, self.H, self.W = ndimage._frames_of(target)
        self.tg = target.contiguous()
        self.ix = ndimage._as_device_idxs(idxs, n, self.dev)
        self.n, self.max_val, self.kernel = n, max_val, kernel
        self.lib = _native.lib()
        nb = int(self.lib.cbc_status_bytes())
        self.status = torch.zeros((max(steps, 1), nb), dtype=torch.uint8).pin_memory()
        self.ws = None

    def first(self, lines: torch.Tensor, delta: torch.Tensor) -> torch.Tensor:
        grad = _packed_loss_step(self.tg, lines, self.ix, self.max_val, self.kernel, delta)
        stream = ndimage._current_stream(self.dev)
        ws = ndimage._workspace_raw(self.dev, stream)
        need = ws.last_status.checkpoints_needed if ws.last_status is not None else 0
        self.cap = ws.capacity
        self.ck = max(ws.ck_capacity, 2 * need + 4096)     # room for the lines to move
        nbytes = self.lib.cbc_squared_loss_step_workspace_size(self.F, self.H, self.W, self.n,
                                                               self.cap, self.ck)
        self.buf = ws.ensure(nbytes)
        self.stream = stream
        return grad

    def enqueue(self, i: int, lines: torch.Tensor, grad: torch.Tensor,
                delta: torch.Tensor) -> None:
        packed = ndimage._packed_scratch(self.dev, self.F * self.H * self.W)
        ix = self.ix
        rc = self.lib.cbc_squared_loss_step_f32(
            self.tg.data_ptr(), self.F, self.H, self.W, lines.data_ptr(), self.n,
            None if ix is None else ix.data_ptr(), 0 if ix is None else ix.element_size(),
            self.max_val, self.k, packed.data_ptr(), grad.data_ptr(), delta.data_ptr(),
            self.buf.data_ptr(), self.buf.numel(), self.cap, self.ck, self.stream)
        if rc == 0:
            rc = self.lib.cbc_copy_status_async(self.buf.data_ptr(), self.status[i].data_ptr(),
                                                self.stream)
        if rc:
            ndimage._raise_rc(rc)

    def failed(self, upto: int) -> bool:
        """after a synchronisation: True if a step in [1, upto) ran out of walk
        checkpoints (it drew nothing); other errors raise"""
        capacity = False
        for i in range(1, upto):
            st = _native.Status()
            self.lib.cbc_decode_status(self.status[i].data_ptr(), st)
            capacity = capacity or st.has(_native.CBC_ERR_CAPACITY)
            ndimage._raise_status(st, self.F)
        return capacity


def squared_loss_step(image: Optional[torch.Tensor], target: torch.Tensor, lines: torch.Tensor,
                      idxs: Optional[torch.Tensor], max_val: float, kernel: str, overlap: str,
                      winner: Optional[torch.Tensor] = None,
                      loss_delta: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Render ``lines`` into ``image`` (overwritten, frames start at zero) and return
    the (N, 5) gradient of sum((image - target)^2): one forward kernel sequence and the
    fused loss adjoint, with no full-frame gradient in memory.  With image None (float32
    max overlap) the forward keeps each pixel's value and winner packed in one scratch
    word, no frames are written, and the adjoint is one pass over those words and the
    target; ``loss_delta`` (float64 CUDA scalar) then receives the loss minus
    sum(target^2)."""
    if image is None:
        if overlap != 'max' or target.dtype != torch.float32:
            raise ValueError("image=None is for float32 max overlap")
        return _packed_loss_step(target, lines, idxs, max_val, kernel, loss_delta)
    if overlap == 'max' and image.dtype == torch.float32:
        # the forward records the winners: no winner pass in the adjoint
        winner = ndimage.draw_lines_max_winner(image, lines, idxs, max_val, kernel, winner)
        return squared_loss_backward(image, target, lines, idxs, max_val, kernel, overlap,
                                     winner=winner, winner_known=True)
    if overlap == 'sum' and image.dtype == torch.float32 and target.dtype == torch.float32 \
            and image.is_cuda and image.is_contiguous():
        return _sum_loss_step(image, target, lines, idxs, max_val, kernel)
    image.zero_()
    ndimage.draw_lines(image, lines, idxs, max_val, kernel, overlap)
    return squared_loss_backward(image, target, lines, idxs, max_val, kernel, overlap,
                                 winner=winner)


def adam_step(params: torch.Tensor, grad: torch.Tensor, exp_avg: torch.Tensor,
              exp_avg_sq: torch.Tensor, step: int, lr: float, betas=(0.9, 0.999),
              eps: float = 1e-8, min_width: float = 0.0) -> None:
    """One Adam step on contiguous float32 CUDA (N, 5) line parameters in place
    (cbc_adam_step_f32: torch.optim.Adam's update, then widths >= min_width); exp_avg
    and exp_avg_sq are the optimiser state (zeros before step 1)."""
    ts = (params, grad, exp_avg, exp_avg_sq)
    if not all(t.is_cuda and t.dtype == torch.float32 and t.is_contiguous() and
               t.shape == params.shape for t in ts) or params.dim() != 2 or params.shape[1] != 5:
        raise ValueError("adam_step takes contiguous float32 CUDA (N, 5) tensors")
    lib = _native.lib()
    with ndimage._on_current_device(params.device):
        rc = lib.cbc_adam_step_f32(params.data_ptr(), grad.data_ptr(), exp_avg.data_ptr(),
                                   exp_avg_sq.data_ptr(), params.shape[0], step, lr, betas[0],
                                   betas[1], eps, min_width,
                                   ndimage._current_stream(params.device))
    if rc:
        ndimage._raise_rc(rc)


def fit_lines(target: torch.Tensor, lines0: torch.Tensor, idxs: Optional[torch.Tensor] = None,
              *, max_val: float = 1.0, kernel: str = 'biweight', overlap: str = 'sum',
              steps: int = 100, lr: float = 0.05, min_width: float = 0.5,
              fused: bool = True, _checked: bool = False) -> FitResult:
    """Refine ``lines0`` (N, 5) so that draw_lines(lines) matches ``target`` (frames on
    the GPU), with ``steps`` Adam steps of learning rate ``lr``.  ``fused`` takes the
    gradient from the fused squared-loss adjoint (squared_loss_step); otherwise it goes
    through torch autograd (draw_lines_fn and a torch loss), with the same result.

    On the float32 max-overlap path the steps after the first do not wait for the GPU:
    their status is read after the last step, and if one of them ran out of walk
    checkpoints (the lines grew far beyond the reserve) the whole fit runs again with a
    check after every step."""
    if not target.is_cuda:
        raise ValueError("target must be a CUDA tensor")
    params = lines0.detach().to(target.device, target.dtype).clone().requires_grad_(True)
    # the fused float32 paths update in one library kernel (cbc_adam_step_f32, torch's
    # Adam formula with its default betas and eps); the others use torch.optim.Adam
    native = fused and target.dtype == torch.float32
    opt = None if native else torch.optim.Adam([params], lr=lr)
    if native:
        exp_avg = torch.zeros_like(params, memory_format=torch.contiguous_format)
        exp_avg_sq = torch.zeros_like(exp_avg)
    with torch.no_grad():
        first = float(_loss(params, idxs, target, max_val, kernel, overlap))
    packed_path = fused and overlap == 'max' and target.dtype == torch.float32
    image = torch.empty_like(target) if fused and not packed_path else None
    winner = (torch.empty(target.shape, dtype=torch.int32, device=target.device)
              if fused and overlap == 'max' and not packed_path else None)
    deltas = torch.zeros(steps, dtype=torch.float64, device=target.device) if packed_path \
        else None
    stepper = (_PackedSteps(target, idxs, max_val, kernel, params.shape[0], steps)
               if packed_path and not _checked else None)
    torch.cuda.synchronize(target.device)
    t0 = time.perf_counter()
    for i in range(steps):
        if stepper is not None and i > 0:
            stepper.enqueue(i, params.detach(), params.grad, deltas[i])
        elif stepper is not None:
            params.grad = stepper.first(params.detach(), deltas[i])
        elif packed_path:
            params.grad = _packed_loss_step(target, params.detach(), idxs, max_val, kernel,
                                            deltas[i])
        elif fused:
            params.grad = squared_loss_step(image, target, params.detach(), idxs, max_val,
                                            kernel, overlap, winner)
        else:
            loss = _loss(params, idxs, target, max_val, kernel, overlap)
            opt.zero_grad(set_to_none=True)
            loss.backward()
        if native:
            adam_step(params.detach(), params.grad, exp_avg, exp_avg_sq, i + 1, lr,
                      min_width=min_width)
        else:
            opt.step()
            with torch.no_grad():
                params[:, 4].clamp_(min=min_width)
    torch.cuda.synchronize(target.device)
    seconds = time.perf_counter() - t0
    if stepper is not None and stepper.failed(steps):
        return fit_lines(target, lines0, idxs, max_val=max_val, kernel=kernel, overlap=overlap,
                         steps=steps, lr=lr, min_width=min_width, fused=fused, _checked=True)
    history = None
    if deltas is not None:
        t2 = float(target.double().pow(2).sum())
        history = [t2 + d for d in deltas.tolist()]
    with torch.no_grad():
        last = float(_loss(params, idxs, target, max_val, kernel, overlap))
    return FitResult(params.detach(), steps, seconds, [first, last], history)


@dataclass
class ShardedFit:
    shard: 'object'                      # shard.Shard: this rank's frames and lines
    result: FitResult                    # this rank's fit (its lines only)
    losses: List[float]                  # loss of the whole stack before and after


def shard_problem(target, lines0, frame_offsets, rank: int, world: int):
    """This rank's part of a streak fit over one stack whose lines are grouped by
    frame (CSR ``frame_offsets``): its contiguous frame range balanced by line counts
    (shard.shard_of), the target frames and lines of that range, and frame indices
    rebased to its first frame.  Host logic only; returns (shard, target, lines,
    idxs)."""
    import numpy as np
    from . import shard as _shard
    offs = np.asarray(torch.as_tensor(frame_offsets).cpu(), dtype=np.int64).reshape(-1)
    sh = _shard.shard_of(offs, rank, world)
    local_t = target[sh.f0:sh.f1]
    local_l = lines0[sh.l0:sh.l1]
    counts = np.diff(sh.local_offsets(offs))
    idxs = torch.from_numpy(np.repeat(np.arange(sh.n_frames, dtype=np.int32), counts))
    return sh, local_t, local_l, idxs


def reduce_losses(losses: List[float]) -> List[float]:
    """sum of every rank's scalar losses (the only cross-rank values of a sharded fit),
    over the default process group when one is initialised"""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return list(losses)
    dev = (torch.device('cuda', torch.cuda.current_device())
           if dist.get_backend() == 'nccl' else torch.device('cpu'))
    t = torch.tensor(losses, dtype=torch.float64, device=dev)
    dist.all_reduce(t)
    return [float(x) for x in t.cpu()]


def fit_lines_sharded(target, lines0, frame_offsets, rank: Optional[int] = None,
                      world: Optional[int] = None, **kw) -> ShardedFit:
    """fit_lines over one stack split across ranks by frames (one process per GPU):
    each rank fits only the lines of its own frames against its own target frames, on
    its current CUDA device; nothing is exchanged on the data path, only the two
    scalar losses are summed.  ``rank``/``world`` default to the default process
    group's (0 and 1 without one).  ``target`` may be a host or device tensor of the
    whole stack; only this rank's frames are moved to the device."""
    import torch.distributed as dist
    if rank is None or world is None:
        if dist.is_available() and dist.is_initialized():
            rank, world = dist.get_rank(), dist.get_world_size()
        else:
            rank, world = 0, 1
    sh, t, ln, ix = shard_problem(target, lines0, frame_offsets, rank, world)
    dev = torch.device('cuda', torch.cuda.current_device())
    res = fit_lines(t.to(dev), ln.to(dev), ix.to(dev), **kw)
    return ShardedFit(sh, res, reduce_losses(res.losses))
