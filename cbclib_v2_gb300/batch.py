"""Ragged frame stacks rendered by one CUDA-graph launch.

A ``RaggedRenderer`` owns device buffers for one stack layout: the frames, the lines
(grouped by frame, CSR ``frame_offsets``) and the library workspace.  Its first call
runs the draw eagerly to size the workspace exactly (plus a margin), picks the render
configuration with the autotuner unless one is given, and captures the whole draw
(the library's kernel sequence for cbc_draw_lines_csr_*) into a CUDA graph; every
call then copies the new lines in and replays the graph, with no host round trip.
``check()`` reads the call's status and re-captures with more room if a later line
set produced more walk checkpoints or (line, tile) pairs than the graph reserved.
"""
import math
from typing import Dict, Optional, Sequence

import torch

from . import _native, autotune, ndimage

__all__ = ['RaggedRenderer', 'render_per_frame']


class RaggedRenderer:
    def __init__(self, shape: Sequence[int], frame_offsets, *, max_val: float = 1.0,
                 kernel: str = 'rectangular', overlap: str = 'sum',
                 dtype: torch.dtype = torch.float32, device=None,
                 tuning: Optional[_native.Tuning] = None, zero: bool = False,
                 margin: float = 1.25, autotune_config: bool = True):
        self.kernel_id, self.overlap_id = ndimage._check_names(kernel, overlap)
        self.kernel, self.overlap, self.max_val = kernel, overlap, float(max_val)
        self.device = torch.device(device or 'cuda')
        self.offsets = torch.as_tensor(frame_offsets).to(self.device, torch.int64).contiguous()
        self.shape = tuple(int(s) for s in shape)
        self.F = math.prod(self.shape[:-2])
        self.H, self.W = self.shape[-2], self.shape[-1]
        if self.offsets.numel() != self.F + 1:
            raise ValueError(f"frame_offsets has {self.offsets.numel()} entries, expected {self.F + 1}")
        self.n_lines = int(self.offsets[-1].item())
        self.dtype = dtype
        self.out = torch.zeros(self.shape, dtype=dtype, device=self.device)
        self.lines = torch.empty((self.n_lines, 5), dtype=dtype, device=self.device)
        self.tuning = tuning
        self.zero = zero
        self.margin = margin
        self.autotune_config = autotune_config and tuning is None
        self.timings: Dict[str, float] = {}
        self.graph: Optional[torch.cuda.CUDAGraph] = None
        self.workspace: Optional[torch.Tensor] = None
        self.capacity = self.ck_capacity = 0

    # -- the captured call ---------------------------------------------------------
    def _call(self, stream_ptr: int) -> int:
        lib = _native.lib()
        fn = lib.cbc_draw_lines_csr_f32 if self.dtype == torch.float32 else lib.cbc_draw_lines_csr_f64
        tref = None if self.tuning is None else ndimage.ctypes_pointer(self.tuning)
        return fn(self.out.data_ptr(), self.F, self.H, self.W, self.lines.data_ptr(), self.n_lines,
                  self.offsets.data_ptr(), self.max_val, self.kernel_id, self.overlap_id,
                  self.workspace.data_ptr(), self.workspace.numel(), self.capacity,
                  self.ck_capacity, tref, stream_ptr)

    def _size_workspace(self):
        """one eager call with the current lines gives the exact capacities"""
        elem = 4 if self.dtype == torch.float32 else 8
        lib = _native.lib()
        cap, ck = 4 * self.n_lines + 1024, 16 * self.n_lines + 1024
        tref = None if self.tuning is None else ndimage.ctypes_pointer(self.tuning)
        stream = torch.cuda.current_stream(self.device)
        for _ in range(4):
            self.capacity, self.ck_capacity = cap, ck
            nbytes = lib.cbc_draw_lines_workspace_size(self.F, self.H, self.W, self.n_lines, cap,
                                                       ck, elem, tref)
            if nbytes == 0:
                raise ValueError(_native.last_error())
            self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            scratch, self.out = self.out, self.out.clone()
            try:
                rc = self._call(stream.cuda_stream)
                if rc:
                    ndimage._raise_rc(rc)
                st = self.status()
            finally:
                self.out = scratch
            ndimage._raise_status(st, self.F)
            if not st.has(_native.CBC_ERR_CAPACITY):
                cap = int(st.pairs_needed * self.margin) + 1024
                ck = int(st.checkpoints_needed * self.margin) + 1024
                self.capacity, self.ck_capacity = cap, ck
                nbytes = lib.cbc_draw_lines_workspace_size(self.F, self.H, self.W, self.n_lines,
                                                           cap, ck, elem, tref)
                self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
                return
            cap = max(cap, int(st.pairs_needed * self.margin) + 1024)
            ck = max(ck, int(st.checkpoints_needed * self.margin) + 1024)
        raise RuntimeError("workspace capacity did not converge")

    def _capture(self):
        self.graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            with torch.cuda.graph(self.graph, stream=side):
                if self.zero:
                    self.out.zero_()
                rc = self._call(side.cuda_stream)
        torch.cuda.current_stream(self.device).wait_stream(side)
        if rc:
            ndimage._raise_rc(rc)

    def prepare(self, lines: torch.Tensor):
        """size the workspace, tune and capture with this line set"""
        with torch.cuda.device(self.device):
            self.lines.copy_(torch.as_tensor(lines).to(self.device, self.dtype).reshape(-1, 5))
            if self.autotune_config:
                self.tuning, self.timings = autotune.tune(
                    self.out, self.lines, None, self.max_val, self.kernel, self.overlap,
                    frame_offsets=self.offsets)
                self.autotune_config = False
            self._size_workspace()
            self._capture()

    def __call__(self, lines: torch.Tensor) -> torch.Tensor:
        """draw `lines` ((n_lines, 5), grouped by frame) into ``self.out`` by one graph
        replay and return ``self.out``"""
        if self.graph is None:
            self.prepare(lines)
        else:
            self.lines.copy_(torch.as_tensor(lines).to(self.device, self.dtype).reshape(-1, 5))
        self.graph.replay()
        return self.out

    def replay(self) -> torch.Tensor:
        """replay with the lines already in ``self.lines``"""
        self.graph.replay()
        return self.out

    def status(self) -> _native.Status:
        st = _native.Status()
        rc = _native.lib().cbc_read_status(self.workspace.data_ptr(), st,
                                           torch.cuda.current_stream(self.device).cuda_stream)
        if rc:
            ndimage._raise_rc(rc)
        return st

    def check(self) -> None:
        """raise the last call's errors; re-capture and replay when it ran out of room"""
        st = self.status()
        ndimage._raise_status(st, self.F)
        if st.has(_native.CBC_ERR_CAPACITY):
            self._size_workspace()
            self._capture()
            self.graph.replay()
            self.check()


def render_per_frame(out: torch.Tensor, lines: torch.Tensor, frame_offsets, max_val: float,
                     kernel: str, overlap: str) -> torch.Tensor:
    """The plain alternative: one public draw_lines call per frame."""
    offs = [int(x) for x in torch.as_tensor(frame_offsets).cpu().tolist()]
    flat = out.reshape(-1, out.shape[-2], out.shape[-1])
    for f in range(flat.shape[0]):
        if offs[f + 1] > offs[f]:
            ndimage.draw_lines(flat[f], lines[offs[f]:offs[f + 1]], None, max_val, kernel, overlap)
    return out
