"""Differentiable draw_lines: gradients of the drawn frames with respect to the line
parameters (x0, y0, x1, y1, width), or (x0, y0, z0, x1, y1, z1, width) for 3-D lines,
from the hand-written adjoint kernels (cbc_draw_lines_backward_*, csrc/cbc_adjoint.cu;
cbc_draw_lines_3d_backward_*, csrc/cbc_lines3d.cu).

``draw_lines_fn(lines, idxs, shape=..., max_val=..., kernel=..., overlap=...)`` returns
new frames ``out0 + draw(lines)`` (``out0`` zeros unless given) and is differentiable
with respect to ``lines`` and ``out0``.  For max overlap the gradient of a pixel goes
to the line whose value the pixel kept (the first in line order among equal values),
or to ``out0`` where no line raised the pixel.
"""
import math
import threading
from typing import Optional, Sequence

import torch

from . import _native, ndimage

__all__ = ['draw_lines_fn', 'DrawLinesFunction', 'lines_backward', 'squared_loss_backward']

_ws_lock = threading.Lock()
_workspaces = {}


def _frames_arg(name: str, t: Optional[torch.Tensor], shape, dtype, dev) -> Optional[torch.Tensor]:
    """`t` as a contiguous `dtype` tensor on `dev` with the frames' number of elements"""
    if t is None:
        return None
    want = math.prod(int(x) for x in shape)
    if t.numel() != want:
        raise ValueError(f"{name} has {t.numel()} elements, the frames {tuple(shape)} have {want}")
    return t.to(device=dev, dtype=dtype).contiguous()


def _check_winner(winner: torch.Tensor, shape, dev) -> None:
    """the winner buffer is written by the kernels: an int32 contiguous CUDA tensor on
    the frames' device with one entry per pixel"""
    want = math.prod(int(x) for x in shape)
    if not (isinstance(winner, torch.Tensor) and winner.dtype == torch.int32 and
            winner.is_contiguous() and winner.numel() == want and winner.device == dev):
        raise ValueError(f"winner must be a contiguous int32 tensor of {want} elements on {dev}")


def _backward(lines, idxs, max_val: float, kernel: str, overlap: str, shape, dtype, dev,
              grad_out: Optional[torch.Tensor] = None, image: Optional[torch.Tensor] = None,
              out0: Optional[torch.Tensor] = None, winner: Optional[torch.Tensor] = None,
              target: Optional[torch.Tensor] = None, winner_known: bool = False,
              packed: Optional[torch.Tensor] = None) -> torch.Tensor:
    """One adjoint call: with grad_out, cbc_draw_lines_backward_*; with target instead,
    cbc_squared_loss_backward_* (grad_out = 2 (image - target) formed per pixel)."""
    k, ov = ndimage._check_names(kernel, overlap)
    if dtype not in (torch.float32, torch.float64):
        raise TypeError(f"frames must be float32 or float64, got {dtype}")
    # every frame-shaped argument covers the frames, so no kernel reads or writes past it
    grad_out = _frames_arg('grad_out', grad_out, shape, dtype, dev)
    image = _frames_arg('image', image, shape, dtype, dev)
    out0 = _frames_arg('out0', out0, shape, dtype, dev)
    target = _frames_arg('target', target, shape, dtype, dev)
    if winner is not None:
        _check_winner(winner, shape, dev)
    ln = ndimage._as_device_lines(lines, dev, dtype)
    if ln.shape[1] == 7:
        if grad_out is None or packed is not None or winner_known:
            raise ValueError("3-D lines take the gradient of the volumes (grad_out)")
        return _backward3(ln, idxs, max_val, k, ov, shape, dtype, dev, grad_out, image, out0,
                          winner)
    n = ln.shape[0]
    ix = ndimage._as_device_idxs(idxs, n, dev)
    H, W = int(shape[-2]), int(shape[-1])
    F = math.prod(int(s) for s in shape[:-2])
    img = None if image is None else image.to(dtype).contiguous()
    o0 = None if out0 is None else out0.to(dtype).contiguous()
    if ov == _native.OVERLAPS['max'] and packed is None:
        if img is None:
            raise ValueError("max overlap needs the forward image")
        if winner is None:
            winner = torch.empty(tuple(shape), dtype=torch.int32, device=dev)
    grad = torch.empty((n, 5), dtype=dtype, device=dev)
    lib = _native.lib()
    elem = 4 if dtype == torch.float32 else 8
    sfx = 'f32' if elem == 4 else 'f64'
    g = None if grad_out is None else grad_out.contiguous()
    tg = None if target is None else target.to(dtype).contiguous()
    if g is None and (tg is None or (img is None and packed is None)):
        raise ValueError("give grad_out, or the forward image and a target")
    fn = getattr(lib, 'cbc_draw_lines_backward_ex_' + sfx)

    def call(buf, ck_capacity, stream):
        return fn(None if g is None else g.data_ptr(), None if tg is None else tg.data_ptr(),
                  F, H, W, ln.data_ptr(), n,
                  None if ix is None else ix.data_ptr(), 0 if ix is None else ix.element_size(),
                  max_val, k, ov, None if img is None else img.data_ptr(),
                  None if o0 is None else o0.data_ptr(),
                  None if winner is None else winner.data_ptr(), int(bool(winner_known)),
                  None if packed is None else packed.data_ptr(),
                  grad.data_ptr(), buf.data_ptr(), buf.numel(), ck_capacity, stream)
    with ndimage._on_current_device(dev):
        stream = ndimage._current_stream(dev)
        key = ('adjoint', dev.index, stream, threading.get_ident())
        ws = _workspaces.get(key)
        if ws is None:
            with _ws_lock:
                ws = _workspaces.setdefault(key, ndimage.Workspace(dev))
        ck_capacity = max(ws.ck_capacity, 16 * n + 1024)
        for _ in range(4):
            nbytes = lib.cbc_draw_lines_backward_workspace_size(n, ck_capacity, elem)
            buf = ws.ensure(nbytes)
            rc = call(buf, ck_capacity, stream)
            if rc:
                ndimage._raise_rc(rc)
            st = _native.Status()
            if lib.cbc_read_status(buf.data_ptr(), st, stream):
                ndimage._raise_rc(_native.CBC_ERR_CUDA)
            ndimage._raise_status(st, F)
            if not st.has(_native.CBC_ERR_CAPACITY):
                ws.ck_capacity = ck_capacity
                return grad
            ck_capacity = max(ck_capacity, int(st.checkpoints_needed * 1.25) + 1024)
    raise RuntimeError("checkpoint capacity did not converge")


def _backward3(ln, idxs, max_val: float, k: int, ov: int, shape, dtype, dev,
               grad_out: torch.Tensor, image: Optional[torch.Tensor],
               out0: Optional[torch.Tensor], winner: Optional[torch.Tensor]) -> torch.Tensor:
    """cbc_draw_lines_3d_backward_*: the (N, 7) gradient for 3-D lines into volumes
    (..., D, H, W)"""
    if len(shape) < 3:
        raise ValueError("3-D lines draw into volumes (..., D, H, W)")
    D, H, W = (int(x) for x in shape[-3:])
    F = math.prod(int(x) for x in shape[:-3])
    n = ln.shape[0]
    ix = ndimage._as_device_idxs(idxs, n, dev)
    if ix is None and n and F != 1 and F != n:
        raise ValueError(f"idxs has an incompatible size ({n} != {F})")
    g = grad_out.to(dtype).contiguous()
    img = None if image is None else image.to(dtype).contiguous()
    o0 = None if out0 is None else out0.to(dtype).contiguous()
    if ov == _native.OVERLAPS['max']:
        if img is None:
            raise ValueError("max overlap needs the forward image")
        if winner is None:
            winner = torch.empty(tuple(shape), dtype=torch.int32, device=dev)
    grad = torch.empty((n, 7), dtype=dtype, device=dev)
    lib = _native.lib()
    elem = 4 if dtype == torch.float32 else 8
    fn = getattr(lib, 'cbc_draw_lines_3d_backward_' + ('f32' if elem == 4 else 'f64'))
    ndimage._run3(
        lambda buf, ck, _t, stream: fn(
            g.data_ptr(), F, D, H, W, ln.data_ptr(), n,
            None if ix is None else ix.data_ptr(), 0 if ix is None else ix.element_size(),
            max_val, k, ov, None if img is None else img.data_ptr(),
            None if o0 is None else o0.data_ptr(), None if winner is None else winner.data_ptr(),
            grad.data_ptr(), buf.data_ptr(), buf.numel(), ck, stream),
        lambda ck, _t: lib.cbc_draw_lines_3d_backward_workspace_size(n, ck, elem),
        dev, 'adjoint3d', F, n, columns=lambda: ndimage._columns3(ln, max(D, H, W)))
    return grad


def lines_backward(grad_out: torch.Tensor, lines: torch.Tensor, idxs: Optional[torch.Tensor],
                   max_val: float, kernel: str, overlap: str,
                   image: Optional[torch.Tensor] = None, out0: Optional[torch.Tensor] = None,
                   winner: Optional[torch.Tensor] = None) -> torch.Tensor:
    """(N, 5) gradient of sum(grad_out * draw_lines(...)) with respect to ``lines``
    ((N, 7) for 3-D lines into volumes).

    ``grad_out`` has the frames' shape and dtype.  Max overlap also needs the forward
    result ``image`` (and ``out0`` if the frames were not zeros); ``winner`` (int32,
    frames' shape) is filled with each pixel's winning line when given."""
    return _backward(lines, idxs, max_val, kernel, overlap, grad_out.shape, grad_out.dtype,
                     grad_out.device, grad_out=grad_out, image=image, out0=out0, winner=winner)


def squared_loss_backward(image: torch.Tensor, target: torch.Tensor, lines: torch.Tensor,
                          idxs: Optional[torch.Tensor], max_val: float, kernel: str,
                          overlap: str, out0: Optional[torch.Tensor] = None,
                          winner: Optional[torch.Tensor] = None,
                          winner_known: bool = False) -> torch.Tensor:
    """(N, 5) gradient of sum((image - target)^2) with respect to ``lines``, where
    ``image = out0 + draw_lines(lines, ...)`` is the forward result (``out0`` None:
    zeros).  The adjoint kernels form 2 (image - target) at each drawn pixel, so no
    full-frame gradient is stored (the fused loss step of a streak fit).  With
    ``winner_known``, ``winner`` holds the forward's winners (draw_lines_max_winner) and
    the winner pass is skipped."""
    return _backward(lines, idxs, max_val, kernel, overlap, image.shape, image.dtype,
                     image.device, image=image, out0=out0, winner=winner, target=target,
                     winner_known=winner_known)


class DrawLinesFunction(torch.autograd.Function):
    """frames = out0 + draw_lines(lines); gradients for lines and out0."""

    @staticmethod
    def forward(ctx, lines, out0, idxs, max_val, kernel, overlap, zero_base=False):
        k, ov = ndimage._check_names(kernel, overlap)
        ctx.meta = (max_val, kernel, overlap)
        ctx.winner = None
        if overlap == 'max' and zero_base and out0.dtype == torch.float32 and \
                lines.shape[-1] == 5:
            # the forward records each pixel's winner: the adjoint skips its winner pass
            image = torch.empty_like(out0, memory_format=torch.contiguous_format)
            ctx.winner = ndimage.draw_lines_max_winner(image, lines.detach(), idxs, max_val,
                                                       kernel)
            ctx.save_for_backward(lines.detach(), idxs, image, None)
            return image
        image = out0.detach().clone(memory_format=torch.contiguous_format)
        ndimage._draw_lines_cuda(image, lines.detach(), idxs, max_val, k, ov)
        if overlap == 'max':
            # frames that started at zero need no out0 in the winner pass
            ctx.save_for_backward(lines.detach(), idxs, image,
                                  None if zero_base else out0.detach())
        else:
            ctx.save_for_backward(lines.detach(), idxs)
        return image

    @staticmethod
    def backward(ctx, grad_image):
        max_val, kernel, overlap = ctx.meta
        saved = ctx.saved_tensors
        lines, idxs = saved[0], saved[1]
        grad_lines = grad_out0 = None
        g = grad_image.contiguous()
        if overlap == 'max':
            image, out0 = saved[2], saved[3]
            known = ctx.winner is not None
            winner = ctx.winner if known else torch.empty(g.shape, dtype=torch.int32,
                                                          device=g.device)
            if ctx.needs_input_grad[0] or not known:
                gl = _backward(lines, idxs, max_val, kernel, overlap, g.shape, g.dtype, g.device,
                               grad_out=g, image=image, out0=out0, winner=winner,
                               winner_known=known)
                if ctx.needs_input_grad[0]:
                    grad_lines = gl
            if ctx.needs_input_grad[1]:
                grad_out0 = torch.where(winner == _native.NO_WINNER, g, torch.zeros_like(g))
        else:
            if ctx.needs_input_grad[0]:
                grad_lines = lines_backward(g, lines, idxs, max_val, kernel, overlap)
            if ctx.needs_input_grad[1]:
                grad_out0 = g
        if grad_lines is not None:
            grad_lines = grad_lines.to(lines.dtype).reshape(lines.shape)
        return grad_lines, grad_out0, None, None, None, None, None


def draw_lines_fn(lines: torch.Tensor, idxs: Optional[torch.Tensor] = None, *,
                  shape: Optional[Sequence[int]] = None, out0: Optional[torch.Tensor] = None,
                  max_val: float = 1.0, kernel: str = 'rectangular',
                  overlap: str = 'sum') -> torch.Tensor:
    """New frames ``out0 + draw_lines(lines)``, differentiable in ``lines`` (N, 5), or
    (N, 7) for 3-D lines into volumes, and ``out0``.  Give either ``shape`` (frames start
    at zero) or ``out0``."""
    zero_base = out0 is None
    if out0 is None:
        if shape is None:
            raise ValueError("give shape or out0")
        out0 = torch.zeros(tuple(shape), dtype=lines.dtype, device=lines.device)
    if lines.shape[-1] not in (5, 7):
        raise RuntimeError(f"Invalid lines size ({lines.shape[-1]}) at axis {lines.ndim - 1}")
    ndimage._check_names(kernel, overlap)
    return DrawLinesFunction.apply(lines, out0, idxs, float(max_val), kernel, overlap, zero_base)
