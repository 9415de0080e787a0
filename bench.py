#!/usr/bin/env python
"""Benchmark of draw_lines on the detector-stack workload (64 frames of 2167x2070
float32, Poisson(2,000) segments per frame, gaussian profile, max overlap, int32 frame
indices): one step = one draw_lines call over the whole stack.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  `value` is device-resident throughput in Mlines/s
(lines, indices and frames already in HBM); `e2e` is the same metric through the
public API with the frames, lines and indices in pinned host buffers: every step copies
the lines and indices to the device, and the kernels combine the drawn pixels into the
host frames in place through their device mapping (only drawn pixels cross the link).  `roofline` is the dominant kernel's achieved HBM bandwidth
(segments_kernel or render_kernel, whichever strategy the call ran) from CUDA events
recorded on its stream around every launch in the timed region.  Its byte count is the
call's contract: draw_lines updates `out` in place, so every output pixel is read and
written once, plus 24 bytes per line (2*F*H*W*4 + 24*N); `write_once_frac` is the same
for an output known to be zero, and `sparse_model` counts only the 32-byte sectors that
hold a drawn pixel (the kernel never touches the others).  `gpu_launches` is the library's own count of
the kernels it launched in the timed region.  `cpu_baseline`
times the oracle (C port of the reference CPU rasteriser) on a bounded sample with
all host threads.  Under torchrun each rank renders its own stack (weak scaling, no
collective on the data path).  `--impl reference` times the reference CPU algorithm
(the oracle port; the reference sources are not on the GPU host) instead.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FALLBACK_HBM_GBS = 6800.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=1000)
    p.add_argument('--warmup', type=int, default=3)
    p.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    p.add_argument('--frames', type=int, default=64)
    p.add_argument('--cpu-frames', type=int, default=0,
                   help='frames in the CPU-baseline sample (0: the whole stack); the '
                        'reference arm sizes its per-step sample to finish in about a '
                        'minute unless this is set')
    p.add_argument('--no-cpu-baseline', action='store_true')
    p.add_argument('--no-e2e', action='store_true')
    p.add_argument('--workload', default='detector_stack',
                   choices=['detector_stack', 'fit', 'ragged', 'fit_loop', 'rotomap',
                            'accumulate2d', 'f64'],
                   help='detector_stack: the headline forward; fit: forward + adjoint '
                        'iterations on 8 x 1024^2 frames vs a finite-difference gradient; '
                        'ragged: 256 x 1024^2 frames with lognormal line counts, one '
                        'CUDA-graph launch vs per-frame plain launches; fit_loop: 100 '
                        'Adam steps of the streak fit on 32 x 2167x2070 frames, 160k '
                        'biweight lines, max overlap; rotomap: 3-D accumulate_lines as '
                        'the indexer calls it (4 x 96^3 volumes, 16k lines, max in a '
                        'streak, sum over streaks); accumulate2d: 2-D accumulate_lines '
                        'with mixed overlaps (16 x 1024^2, 64k lines); f64: the detector '
                        'stack in float64')
    args = p.parse_args()
    args.steps_given = any(a == '--steps' or a.startswith('--steps=') for a in sys.argv[1:])
    args.frames_given = any(a == '--frames' or a.startswith('--frames=') for a in sys.argv[1:])
    return args


def dist_env():
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 100 ms; only the samples taken
    between begin() and end() (the timed region) are reported."""
    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.window = (0.0, float('inf'))

    def start(self):
        """start sampling and wait (at most 10 s) for the first sample"""
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', f'--query-gpu={self.FIELDS}', '--format=csv,noheader,nounits',
                 '-lms', '100', '-i', str(self.gpu)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (OSError, ValueError):
            self.proc = None
            return
        t_end = time.perf_counter() + 10.0
        while not self.lines and time.perf_counter() < t_end and self.proc.poll() is None:
            time.sleep(0.01)

    def begin(self):
        self.window = (time.perf_counter(), float('inf'))

    def end(self):
        self.window = (self.window[0], time.perf_counter())

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        lo, hi = self.window
        for t, ln in self.lines:
            if not lo <= t <= hi:
                continue
            f = [x.strip() for x in ln.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith('active'):
                    reasons.add(n)
        return {'sm_mhz': statistics.median(sm) if sm else None,
                'sm_max_mhz': max(smax) if smax else None,
                'reasons': sorted(reasons), 'samples': len(sm)}


def measured_peak():
    path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    try:
        with open(path) as fh:
            return float(json.load(fh)['hbm_gbs']), 'measured'
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, 'fallback'


def committed_traffic(workload: str, kernel: str):
    """DRAM bytes (read + write) per launch of `kernel` on `workload` from the committed
    ncu summary, or None."""
    path = os.path.join(ROOT, 'profiles', 'render_traffic.json')
    try:
        with open(path) as fh:
            d = json.load(fh)
        return d.get(workload, {}).get(kernel)
    except (OSError, ValueError, AttributeError):
        return None


def cpu_baseline(ls, n_frames: int, repeats: int = 3):
    """The oracle (reference CPU algorithm, C port) on the first frames, all threads."""
    import oracle
    from cbclib_v2_gb300 import workloads
    n_frames = ls.shape[0] if n_frames <= 0 else min(n_frames, ls.shape[0])
    sub = workloads.frames_subset(ls, list(range(n_frames)))
    lines = sub.lines.astype(np.float32)
    threads = len(os.sched_getaffinity(0))
    best = float('inf')
    for _ in range(repeats):
        out = np.zeros(sub.shape, np.float32)
        t0 = time.perf_counter()
        oracle.draw_lines(out, lines, sub.idxs, sub.max_val, sub.kernel, sub.overlap, threads)
        best = min(best, time.perf_counter() - t0)
    return {'value': sub.n_lines / best / 1e6, 'unit': 'Mlines/s', 'cores': threads,
            'kind': 'port', 'seconds': best, 'lines': sub.n_lines,
            'sample': f'{sub.shape[0]} of {ls.shape[0]} frames ({sub.n_lines} lines), '
                      f'best of {repeats}'}


def run_reference(args, ls, world, rank):
    if rank != 0:
        return
    import oracle  # noqa: F401  (builds the C port on first use)
    cfg = workload_config(ls)
    frames = args.cpu_frames
    for _ in range(max(args.warmup, 1)):
        probe = cpu_baseline(ls, 2, repeats=1)
    if frames <= 0:
        # about 60 s of CPU work over all timed steps, at least one frame per step
        per_frame = probe['seconds'] / 2
        frames = int(min(ls.shape[0], max(1, round(60.0 / max(args.steps, 1) / per_frame))))
    vals = []
    for _ in range(args.steps):
        vals.append(cpu_baseline(ls, frames, repeats=1))
    secs = sum(v['seconds'] for v in vals)
    lines = sum(v['lines'] for v in vals)
    value = lines / secs / 1e6
    cb = dict(vals[0])
    cb['value'] = value
    cb['sample'] = f'the first {frames} of {ls.shape[0]} frames per step'
    cb.pop('seconds', None)
    cb.pop('lines', None)
    print(json.dumps({
        'impl': 'reference', 'metric': 'draw_lines throughput', 'value': value,
        'unit': 'Mlines/s', 'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': secs / args.steps * 1e3, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic', 'config': cfg,
        'cpu_baseline': cb,
        'e2e': {'value': value, 'unit': 'Mlines/s', 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': 0}}), flush=True)


def workload_config(ls):
    F, H, W = ls.shape
    return {'workload': ls.name, 'frames': F, 'height': H, 'width': W, 'lines': ls.n_lines,
            'kernel': ls.kernel, 'overlap': ls.overlap, 'idx_dtype': 'int32',
            'out_dtype': 'float32', 'contract': 'read-modify-write of out',
            'l2': 'output frames (%.2f GB) exceed L2; no flush' % (F * H * W * 4 / 1e9)}


def run_fit(args, world, rank, local):
    """forward + loss + adjoint iterations/s on the 8 x 1024^2 workload, next to the
    cost of a finite-difference gradient from the plain forward (2 forwards per
    parameter, 5 parameters per line)"""
    import torch
    from cbclib_v2_gb300 import _native, autograd, draw_lines, fit, workloads
    torch.cuda.set_device(local)
    ls = workloads.fit_stack(seed=2000 + rank)
    truth = torch.from_numpy(ls.lines.astype(np.float32)).cuda()
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).cuda()
    target = torch.zeros(ls.shape, device='cuda')
    draw_lines(target, workloads.perturbed(ls.lines, 7).astype(np.float32), ls.idxs,
               ls.max_val, ls.kernel, ls.overlap)
    gen = torch.Generator(device='cuda').manual_seed(3)
    target = torch.poisson(target, generator=gen)
    params = truth.clone().requires_grad_(True)

    def step():
        img = autograd.draw_lines_fn(params, idxs, shape=ls.shape, max_val=ls.max_val,
                                     kernel=ls.kernel, overlap=ls.overlap)
        loss = ((img - target) ** 2).sum()
        params.grad = None
        loss.backward()
        return loss

    image = torch.empty_like(target)

    def fused_step():
        return fit.squared_loss_step(image, target, truth, idxs, ls.max_val, ls.kernel,
                                     ls.overlap)

    stream = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(args.steps):
            r = fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / args.steps, r

    ms_iter, _ = timed(fused_step)                 # forward + fused loss adjoint
    ms_autograd, loss = timed(step)                # torch autograd and a torch loss
    # one plain forward, the unit of a finite-difference gradient
    out = torch.zeros(ls.shape, device='cuda')
    for _ in range(3):
        out.zero_()
        draw_lines(out, truth, idxs, ls.max_val, ls.kernel, ls.overlap)
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(args.steps):
        out.zero_()
        draw_lines(out, truth, idxs, ls.max_val, ls.kernel, ls.overlap)
    b.record(stream)
    torch.cuda.synchronize()
    ms_fwd = a.elapsed_time(b) / args.steps
    fd_ms = 2 * 5 * ls.n_lines * ms_fwd
    if rank == 0:
        print(json.dumps({
            'metric': 'forward+adjoint iterations/s', 'value': 1e3 / ms_iter * world,
            'unit': 'iter/s', 'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': ms_iter, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': ls.name, 'frames': ls.shape[0], 'lines': ls.n_lines,
                       'kernel': ls.kernel, 'overlap': ls.overlap,
                       'loss': 'sum((I - target)^2), target = Poisson(render(perturbed))'},
            'path': 'fused: draw_lines + squared-loss adjoint (2 (I - T) per drawn pixel)',
            'autograd_ms_per_iter': ms_autograd,
            'forward_ms': ms_fwd,
            'finite_difference_gradient_ms': fd_ms,
            'speedup_vs_finite_difference': fd_ms / ms_iter,
            'loss': float(loss.item())}), flush=True)


def run_ragged(args, world, rank, local):
    """256 frames of 1024^2, lognormal(median 1,500, sigma 1) segments per frame clipped
    to [100, 20,000], triangular, sum: one graph replay of the autotuned CSR draw per
    step, against one public draw_lines call per frame"""
    import torch
    from cbclib_v2_gb300 import batch, workloads
    torch.cuda.set_device(local)
    ls = workloads.ragged_stack(seed=3000 + rank)
    offs = ls.frame_offsets()
    lines = torch.from_numpy(ls.lines.astype(np.float32)).cuda()
    r = batch.RaggedRenderer(ls.shape, offs, max_val=ls.max_val, kernel=ls.kernel,
                             overlap=ls.overlap)
    r(lines)
    r.check()
    for _ in range(args.warmup):
        r.replay()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(args.steps):
        r.replay()
    b.record(stream)
    torch.cuda.synchronize()
    ms_graph = a.elapsed_time(b) / args.steps
    r.check()
    out = torch.zeros(ls.shape, device='cuda')
    batch.render_per_frame(out, lines, offs, ls.max_val, ls.kernel, ls.overlap)
    torch.cuda.synchronize()
    k = max(2, args.steps // 5)
    a.record(stream)
    for _ in range(k):
        batch.render_per_frame(out, lines, offs, ls.max_val, ls.kernel, ls.overlap)
    b.record(stream)
    torch.cuda.synchronize()
    ms_frames = a.elapsed_time(b) / k
    t = r.tuning
    if rank == 0:
        print(json.dumps({
            'metric': 'ragged draw_lines throughput', 'value': world * ls.n_lines / ms_graph / 1e3,
            'unit': 'Mlines/s', 'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': ms_graph, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': ls.name, 'frames': ls.shape[0], 'lines': ls.n_lines,
                       'lines_per_frame_min_max': [int(np.diff(offs).min()), int(np.diff(offs).max())],
                       'kernel': ls.kernel, 'overlap': ls.overlap},
            'autotuned': {f: getattr(t, f) for f, _ in type(t)._fields_} if t is not None else None,
            'autotune_ms': r.timings,
            'per_frame_launches_ms': ms_frames,
            'graph_speedup_vs_per_frame': ms_frames / ms_graph}), flush=True)


def _device_steps(fn, args, local):
    """W untimed calls, then K calls between CUDA events on the current stream, with
    the clocks sampled in between; returns (ms per call, clocks)"""
    import torch
    for _ in range(max(args.warmup, 1)):
        fn()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    stream = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks.begin()
    a.record(stream)
    for _ in range(args.steps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    clocks.end()
    return a.elapsed_time(b) / args.steps, clocks.stop()


def run_accumulate(args, world, rank, local):
    """accumulate_lines throughput (device-resident), next to the oracle's CPU
    accumulate_lines (terms shared out among all host threads, as the reference does,
    bresenham.cpp:151-259) on the first frames"""
    import torch
    import oracle
    from cbclib_v2_gb300 import _native, accumulate_lines, workloads
    torch.cuda.set_device(local)
    ts = (workloads.rotomap_stack(seed=5000 + rank) if args.workload == 'rotomap'
          else workloads.accumulate_stack(seed=5100 + rank))
    dev = torch.device('cuda', local)
    lines = torch.from_numpy(ts.lines.astype(np.float32)).to(dev)
    terms = torch.from_numpy(ts.terms.astype(np.int32)).to(dev)
    frames = torch.from_numpy(ts.frames.astype(np.int32)).to(dev)
    out = torch.zeros(ts.shape, dtype=torch.float32, device=dev)

    def step():
        accumulate_lines(out, lines, terms, frames, ts.max_val, ts.kernel, ts.in_overlap,
                         ts.out_overlap)

    _native.profile_enable(True)
    _native.profile_read(reset=True)
    ms, clocks = _device_steps(step, args, local)
    prof = _native.profile_read(reset=True)
    _native.profile_enable(False)
    cb = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = len(os.sched_getaffinity(0))
        k = 1
        sub = ts.subset(k)
        while True:
            o = np.zeros(sub.shape, np.float32)
            t0 = time.perf_counter()
            oracle.accumulate_lines(o, sub.lines.astype(np.float32), sub.terms, sub.frames,
                                    sub.max_val, sub.kernel, sub.in_overlap, sub.out_overlap,
                                    threads)
            sec = time.perf_counter() - t0
            if sec > 5.0 or k >= ts.shape[0]:
                break
            k = min(ts.shape[0], k * 2)
            sub = ts.subset(k)
        cb = {'value': sub.n_lines / sec / 1e6, 'unit': 'Mlines/s', 'cores': threads,
              'kind': 'port',
              'sample': f'{k} of {ts.shape[0]} frames ({sub.n_lines} lines), one run'}
    if rank == 0:
        print(json.dumps({
            'metric': 'accumulate_lines throughput', 'value': world * ts.n_lines / ms / 1e3,
            'unit': 'Mlines/s', 'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': ts.name, 'shape': list(ts.shape), 'lines': ts.n_lines,
                       'terms': int(ts.frames.size), 'kernel': ts.kernel,
                       'in_overlap': ts.in_overlap, 'out_overlap': ts.out_overlap,
                       'out': 'accumulated in place, not re-zeroed between steps'},
            'clocks': clocks, 'gpu_launches': prof.launches, 'cpu_baseline': cb}), flush=True)


def run_f64(args, world, rank, local):
    """the detector stack drawn in float64 (lines and frames), device-resident, next to
    the oracle's float64 draw_lines on all host threads"""
    import torch
    import oracle
    from cbclib_v2_gb300 import _native, draw_lines, workloads
    torch.cuda.set_device(local)
    ls = workloads.detector_stack(seed=1000 + rank, F=args.frames)
    dev = torch.device('cuda', local)
    lines = torch.from_numpy(ls.lines.astype(np.float64)).to(dev)
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).to(dev)
    out = torch.zeros(ls.shape, dtype=torch.float64, device=dev)
    _native.profile_enable(True)
    _native.profile_read(reset=True)
    ms, clocks = _device_steps(
        lambda: draw_lines(out, lines, idxs, ls.max_val, ls.kernel, ls.overlap), args, local)
    prof = _native.profile_read(reset=True)
    _native.profile_enable(False)
    F, H, W = ls.shape
    cb = None
    if rank == 0 and not args.no_cpu_baseline:
        sub = workloads.frames_subset(ls, [0, 1])
        o = np.zeros(sub.shape, np.float64)
        threads = len(os.sched_getaffinity(0))
        t0 = time.perf_counter()
        oracle.draw_lines(o, sub.lines, sub.idxs, sub.max_val, sub.kernel, sub.overlap, threads)
        sec = time.perf_counter() - t0
        cb = {'value': sub.n_lines / sec / 1e6, 'unit': 'Mlines/s', 'cores': threads,
              'kind': 'port', 'sample': f'2 of {F} frames ({sub.n_lines} lines), one run'}
    render_ms = prof.ms_render / max(prof.calls, 1)
    contract = 2 * F * H * W * 8 + 44 * ls.n_lines
    peak, src = measured_peak()
    if rank == 0:
        print(json.dumps({
            'metric': 'draw_lines throughput', 'value': world * ls.n_lines / ms / 1e3,
            'unit': 'Mlines/s', 'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f64', 'data': 'synthetic',
            'config': {'workload': ls.name + '_f64', 'frames': F, 'lines': ls.n_lines,
                       'kernel': ls.kernel, 'overlap': ls.overlap, 'out_dtype': 'float64'},
            'roofline': {'bound': 'hbm', 'achieved': contract / (render_ms * 1e-3) / 1e9,
                         'peak': peak, 'peak_source': src, 'unit': 'GB/s',
                         'frac': contract / (render_ms * 1e-3) / 1e9 / peak, 'traffic': None,
                         'bytes_model': '2*F*H*W*8 + 44*N over the render kernel time',
                         'kernel': 'segments_kernel', 'ms_per_launch': render_ms},
            'clocks': clocks, 'gpu_launches': prof.launches, 'cpu_baseline': cb}), flush=True)


def run_fit_loop(args, world, rank, local):
    """the streak-fit loop: 32 frames of 2167x2070, 5,000 biweight lines per frame,
    max overlap; the target is Poisson noise on the render of the true lines (peak 100
    counts), the start is the truth
    perturbed by N(0, 1 px) on the endpoints and N(0, 0.3 px) on the widths; 100 Adam
    steps of lr 0.05 (--steps overrides the count); reports steps/s and the parameter
    RMS against the truth before and after"""
    import torch
    from cbclib_v2_gb300 import draw_lines, fit, workloads
    torch.cuda.set_device(local)
    frames = args.frames if args.frames_given else 32
    ls = workloads.fit_loop_stack(seed=4000 + rank, F=frames)
    dev = torch.device('cuda', local)
    truth = torch.from_numpy(ls.lines.astype(np.float32)).to(dev)
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).to(dev)
    target = torch.zeros(ls.shape, device=dev)
    draw_lines(target, truth, idxs, ls.max_val, ls.kernel, ls.overlap)
    gen = torch.Generator(device=dev).manual_seed(4200 + rank)
    target = torch.poisson(target, generator=gen)          # counts, peak 100 per line
    start = torch.from_numpy(workloads.perturbed(ls.lines, 4100 + rank, 1.0, 0.3)
                             .astype(np.float32)).to(dev)
    steps = args.steps if args.steps_given else 100
    fit.fit_lines(target, start, idxs, max_val=ls.max_val, kernel=ls.kernel,
                  overlap=ls.overlap, steps=max(args.warmup, 1), lr=0.05)      # warm-up
    res = fit.fit_lines(target, start, idxs, max_val=ls.max_val, kernel=ls.kernel,
                        overlap=ls.overlap, steps=steps, lr=0.05)

    def rms(p):
        d = (p - truth).double()
        return {'endpoints_px': float(d[:, :4].pow(2).mean().sqrt()),
                'width_px': float(d[:, 4].pow(2).mean().sqrt())}

    if rank == 0:
        print(json.dumps({
            'metric': 'streak-fit Adam steps/s', 'value': world * 1e3 / res.ms_per_step,
            'unit': 'steps/s', 'n_gpus': world, 'steps': steps, 'warmup': args.warmup,
            'ms_per_step': res.ms_per_step, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': ls.name, 'frames': ls.shape[0], 'lines': ls.n_lines,
                       'kernel': ls.kernel, 'overlap': ls.overlap, 'lr': 0.05,
                       'loss': 'sum((I - T)^2), T = Poisson(render of the true lines), '
                               'peak 100 counts',
                       'start': 'truth + N(0, 1 px) endpoints, N(0, 0.3 px) widths'},
            'rms_start': rms(start), 'rms_final': rms(res.lines),
            'loss_start': res.losses[0], 'loss_final': res.losses[-1]}), flush=True)


def main():
    args = parse()
    world, rank, local = dist_env()
    if args.workload == 'fit_loop' and args.impl == 'gb300':
        run_fit_loop(args, world, rank, local)
        return
    if args.workload in ('rotomap', 'accumulate2d') and args.impl == 'gb300':
        run_accumulate(args, world, rank, local)
        return
    if args.workload == 'f64' and args.impl == 'gb300':
        run_f64(args, world, rank, local)
        return
    if args.workload == 'fit' and args.impl == 'gb300':
        run_fit(args, world, rank, local)
        return
    if args.workload == 'ragged' and args.impl == 'gb300':
        run_ragged(args, world, rank, local)
        return
    import torch
    from cbclib_v2_gb300 import _native, draw_lines, ndimage, workloads

    ls = workloads.detector_stack(seed=1000 + rank, F=args.frames)
    if args.impl == 'reference':
        run_reference(args, ls, world, rank)
        return

    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl', init_method='env://')
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    F, H, W = ls.shape
    N = ls.n_lines
    lines = torch.from_numpy(ls.lines.astype(np.float32)).to(dev)
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).to(dev)
    out = torch.zeros(ls.shape, dtype=torch.float32, device=dev)

    def barrier():
        if dist is not None:
            dist.barrier(device_ids=[local])

    for _ in range(args.warmup):
        draw_lines(out, lines, idxs, ls.max_val, ls.kernel, ls.overlap)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    _native.profile_enable(True)
    _native.profile_read(reset=True)
    barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks.begin()
    t0.record(stream)
    for _ in range(args.steps):
        draw_lines(out, lines, idxs, ls.max_val, ls.kernel, ls.overlap)
    t1.record(stream)
    torch.cuda.synchronize()
    clocks.end()
    barrier()
    prof = _native.profile_read(reset=True)
    strategy = ndimage.last_status(dev).strategy
    _native.profile_enable(False)
    clk = clocks.stop()
    ms = t0.elapsed_time(t1)
    if dist is not None:
        tt = torch.tensor([ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    ms_step = ms / args.steps
    value = world * N / (ms_step * 1e-3) / 1e6

    # end to end through the public API with pinned host buffers
    e2e = None
    if not args.no_e2e:
        h_out = torch.zeros(ls.shape, dtype=torch.float32).pin_memory()
        h_lines = torch.from_numpy(ls.lines.astype(np.float32)).pin_memory()
        h_idxs = torch.from_numpy(ls.idxs.astype(np.int32)).pin_memory()
        for _ in range(max(1, args.warmup)):
            draw_lines(h_out, h_lines, h_idxs, ls.max_val, ls.kernel, ls.overlap)
        e_steps = max(3, min(args.steps // 4, 50))
        barrier()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(e_steps):
            draw_lines(h_out, h_lines, h_idxs, ls.max_val, ls.kernel, ls.overlap)
        b.record(stream)
        torch.cuda.synchronize()
        barrier()
        e_ms = a.elapsed_time(b) / e_steps
        if dist is not None:
            tt = torch.tensor([e_ms], device=dev)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            e_ms = float(tt.item())
        # the frames stay in page-locked host memory: the library's kernels read and
        # write the drawn pixels there through their device mapping (NVLink-C2C), so
        # the bytes across the link per step are the lines and indices up, and the
        # drawn pixels read and written in place (counted from a draw into zeros)
        ref = torch.zeros(ls.shape, dtype=torch.float32, device=dev)
        draw_lines(ref, lines, idxs, ls.max_val, ls.kernel, ls.overlap)
        drawn = int((ref != 0).sum())
        del ref
        e2e = {'value': world * N / (e_ms * 1e-3) / 1e6, 'unit': 'Mlines/s',
               'ms_per_step': e_ms,
               'h2d_bytes_per_step': int(h_lines.numel() * 4 + h_idxs.numel() * 4 + drawn * 4),
               'd2h_bytes_per_step': int(drawn * 4),
               'frames': 'page-locked host memory, drawn pixels combined in place by the '
                         'kernels (zero-copy); %d of %d pixels drawn' % (drawn, h_out.numel())}

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    peak, peak_src = measured_peak()
    render_ms = prof.ms_render / max(prof.calls, 1)
    kname = 'segments_kernel' if strategy == _native.STRATEGY_LINES else 'render_kernel'
    # bytes the op must move: every 32-byte sector of `out` holding a drawn pixel is
    # read and written once (all other sectors are untouched), plus each line's
    # 5 coordinates and frame index
    drawn_sectors = int(out.reshape(-1, 8).ne(0).any(dim=1).sum().item())
    algo_bytes = 64 * drawn_sectors + N * 24
    full_bytes = 2 * F * H * W * 4 + N * 24
    achieved = full_bytes / (render_ms * 1e-3) / 1e9
    sparse = algo_bytes / (render_ms * 1e-3) / 1e9
    roofline = {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                'frac': achieved / peak, 'peak_source': peak_src,
                'traffic': committed_traffic(ls.name, kname), 'kernel': kname,
                'algorithmic_bytes': full_bytes,
                'bytes_model': 'read + write of every output pixel (the call updates out '
                               'in place) + 24 B per line: 2*F*H*W*4 + 24*N',
                'write_once_frac': (full_bytes / 2 + N * 12) / (render_ms * 1e-3) / 1e9 / peak,
                'sparse_model': {'bytes': algo_bytes, 'achieved': sparse,
                                 'frac': sparse / peak,
                                 'model': 'read+write of each 32 B sector holding a drawn '
                                          'pixel (%d of %d sectors) + 24 B per line'
                                          % (drawn_sectors, F * H * W // 8)},
                'ms_per_launch': render_ms,
                'stage_ms_per_call': {
                    'prep': prof.ms_prep / max(prof.calls, 1),
                    'offsets': prof.ms_offsets / max(prof.calls, 1),
                    'fill': prof.ms_fill / max(prof.calls, 1),
                    'render': render_ms}}
    res = {
        'metric': 'draw_lines throughput', 'value': value, 'unit': 'Mlines/s', 'n_gpus': world,
        'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms_step,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
        'data': 'synthetic', 'config': workload_config(ls), 'roofline': roofline,
        'output_gbs': F * H * W * 4 / (ms_step * 1e-3) / 1e9, 'clocks': clk,
        'gpu_launches': prof.launches, 'e2e': e2e,
    }
    if not args.no_cpu_baseline and world == 1:
        cb = cpu_baseline(ls, args.cpu_frames, repeats=2)
        cb.pop('seconds', None)
        cb.pop('lines', None)
        res['cpu_baseline'] = cb
    print(json.dumps(res), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
