#!/usr/bin/env python
"""Benchmark of draw_lines on the detector-stack workload (64 frames of 2167x2070
float32, Poisson(2,000) segments per frame, gaussian profile, max overlap, int32 frame
indices): one step = one draw_lines call over the whole stack.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  `value` is device-resident throughput in Mlines/s
(lines, indices and frames already in HBM).  `e2e` is the same metric through the
public API the reference's callers use: NumPy frames, lines and indices in host
memory; every step copies the lines and indices to the device, and the kernels
combine the drawn pixels into the host frames in place over NVLink-C2C (only drawn
pixels cross the link); `e2e_pinned` is the same with page-locked torch tensors.
`roofline` is the dominant kernel's achieved HBM bandwidth (segments_kernel or
render_kernel, whichever strategy the call ran) from CUDA events recorded on its
stream around every launch in the timed region.  Its byte count is the call's
contract: draw_lines updates `out` in place, so every output pixel is read and written
once, plus 24 bytes per line (2*F*H*W*4 + 24*N); `write_once_frac` is the same for an
output known to be zero, `sparse_model` counts only the 32-byte sectors that hold a
drawn pixel (the kernel never touches the others), and `traffic_frac` is the DRAM
traffic ncu measured for one launch over the launch's time.  `gpu_launches` is the
library's own count of the kernels it launched in the timed region.  `clocks` are
NVML samples (every 2 ms) taken inside the timed region.  `cpu_baseline` times the
oracle (C port of the reference CPU rasteriser) in a fresh process, on all host
threads and on one, with `out` zeroed and touched before the clock.  `workloads`
holds the other benchmark configurations, run after the headline: the
forward+adjoint iterations on 8 x 1024^2 frames against a finite-difference
gradient, the ragged 256 x 1024^2 stack by one CUDA-graph replay, and the
32 x 2167x2070 streak-fit loop.  Under torchrun each rank renders its own stack (weak
scaling, no collective on the data path), or with --shard the ranks split one stack
by frames.  `--impl reference` times the reference CPU algorithm (the oracle port;
the reference sources are not on the GPU host) instead.
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
    p.add_argument('--headline-only', action='store_true',
                   help='skip the other configurations after the headline')
    p.add_argument('--shard', action='store_true',
                   help='under torchrun: split one stack across the ranks by frames '
                        '(balanced by line counts) instead of one stack per rank')
    p.add_argument('--cpu-child', action='store_true', help=argparse.SUPPRESS)
    p.add_argument('--cpu-threads', type=int, default=1, help=argparse.SUPPRESS)
    p.add_argument('--repeats', type=int, default=1, help=argparse.SUPPRESS)
    p.add_argument('--seed', type=int, default=1000, help=argparse.SUPPRESS)
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
    """SM clock, its maximum, power and clock-event reasons of one GPU, sampled every
    2 ms through NVML (libnvidia-ml, ctypes) from start() to stop(); only samples
    taken between begin() and end() (the timed region) are reported.  Falls back to
    `nvidia-smi -lms 100` when NVML cannot be loaded."""
    REASONS = {0x4: 'sw_power_cap', 0x8: 'hw_slowdown', 0x20: 'sw_thermal_slowdown',
               0x40: 'hw_thermal_slowdown', 0x80: 'hw_power_brake_slowdown'}
    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu: int, period_s: float = 0.002):
        self.gpu = gpu
        self.period = period_s
        self.samples = []              # (time, sm MHz, max MHz, reason bits)
        self.window = (0.0, float('inf'))
        self.proc = None
        self.nvml = None
        self.handle = None
        self.stop_flag = threading.Event()
        self.thread = None
        self.source = None

    def _nvml_open(self):
        import ctypes
        try:
            nv = ctypes.CDLL('libnvidia-ml.so.1')
        except OSError:
            return False
        if nv.nvmlInit_v2() != 0:
            return False
        handle = ctypes.c_void_p()
        found = False
        try:
            import torch
            uuid = str(torch.cuda.get_device_properties(self.gpu).uuid)
            found = nv.nvmlDeviceGetHandleByUUID(('GPU-' + uuid).encode(),
                                                 ctypes.byref(handle)) == 0
        except Exception:
            found = False
        if not found:
            found = nv.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.gpu),
                                                     ctypes.byref(handle)) == 0
        if not found:
            return False
        self.nvml, self.handle = nv, handle
        return True

    def _nvml_loop(self):
        import ctypes
        nv, h = self.nvml, self.handle
        sm, mx, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        while not self.stop_flag.is_set():
            ok = (nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(sm)) == 0 and
                  nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0 and
                  nv.nvmlDeviceGetCurrentClocksEventReasons(h, ctypes.byref(rs)) == 0)
            if ok:
                self.samples.append((time.perf_counter(), float(sm.value), float(mx.value),
                                     int(rs.value)))
            time.sleep(self.period)

    def start(self):
        """start sampling and wait (at most 10 s) for the first sample"""
        if self._nvml_open():
            self.source = 'nvml'
            self.thread = threading.Thread(target=self._nvml_loop, daemon=True)
            self.thread.start()
        else:
            try:
                self.proc = subprocess.Popen(
                    ['nvidia-smi', f'--query-gpu={self.FIELDS}', '--format=csv,noheader,nounits',
                     '-lms', '100', '-i', str(self.gpu)], stdout=subprocess.PIPE,
                    stderr=subprocess.DEVNULL, text=True)
                self.source = 'nvidia-smi'
                threading.Thread(target=self._smi_read, daemon=True).start()
            except (OSError, ValueError):
                self.proc = None
                return
        t_end = time.perf_counter() + 10.0
        while not self.samples and time.perf_counter() < t_end:
            if self.proc is not None and self.proc.poll() is not None:
                break
            time.sleep(0.005)

    def _smi_read(self):
        names = {'hw_slowdown': 0x8, 'hw_thermal_slowdown': 0x40, 'sw_thermal_slowdown': 0x20,
                 'sw_power_cap': 0x4}
        for line in self.proc.stdout:
            f = [x.strip() for x in line.strip().split(',')]
            if len(f) < 9:
                continue
            try:
                bits = 0
                for (n, b), v in zip(names.items(), f[5:9]):
                    if v.lower().startswith('active'):
                        bits |= b
                self.samples.append((time.perf_counter(), float(f[1]), float(f[2]), bits))
            except ValueError:
                continue

    def begin(self):
        self.window = (time.perf_counter(), float('inf'))

    def end(self):
        self.window = (self.window[0], time.perf_counter())

    def stop(self):
        if self.thread is not None:
            self.stop_flag.set()
            self.thread.join(timeout=5)
        elif self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        else:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['clock sampling unavailable'],
                    'samples': 0}
        lo, hi = self.window
        sel = [x for x in self.samples if lo <= x[0] <= hi]
        reasons = set()
        for _, _, _, bits in sel:
            for b, n in self.REASONS.items():
                if bits & b:
                    reasons.add(n)
        return {'sm_mhz': statistics.median(x[1] for x in sel) if sel else None,
                'sm_max_mhz': max(x[2] for x in sel) if sel else None,
                'reasons': sorted(reasons), 'samples': len(sel), 'source': self.source,
                'period_ms': self.period * 1e3 if self.source == 'nvml' else 100.0}


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


def cpu_model() -> str:
    """the host CPU's model name (lscpu, else /proc/cpuinfo, else platform)"""
    try:
        out = subprocess.run(['lscpu'], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith('Model name:'):
                return line.split(':', 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open('/proc/cpuinfo') as fh:
            for line in fh:
                if line.lower().startswith('model name'):
                    return line.split(':', 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def time_oracle(ls, n_frames: int, threads: int, repeats: int):
    """best-of-`repeats` seconds of the oracle (the reference CPU algorithm, C port) on
    the first `n_frames` frames with `threads` threads; `out` is allocated and touched
    before the clock starts, so first-touch page faults stay outside the timed region"""
    import oracle
    from cbclib_v2_gb300 import workloads
    n_frames = ls.shape[0] if n_frames <= 0 else min(n_frames, ls.shape[0])
    sub = workloads.frames_subset(ls, list(range(n_frames)))
    lines = sub.lines.astype(np.float32)
    best = float('inf')
    for _ in range(repeats):
        out = np.zeros(sub.shape, np.float32)
        out.fill(0.0)
        t0 = time.perf_counter()
        oracle.draw_lines(out, lines, sub.idxs, sub.max_val, sub.kernel, sub.overlap, threads)
        best = min(best, time.perf_counter() - t0)
    return {'seconds': best, 'lines': sub.n_lines, 'frames': n_frames}


def cpu_child(args):
    """--cpu-child: time_oracle in this fresh process, one JSON line on stdout"""
    from cbclib_v2_gb300 import workloads
    ls = workloads.detector_stack(seed=args.seed, F=args.frames)
    print(json.dumps(time_oracle(ls, args.cpu_frames, args.cpu_threads, args.repeats)),
          flush=True)


def cpu_baseline(args, rank: int):
    """The oracle on the host cores, each measurement in a fresh interpreter (started
    with subprocess, no CUDA context, no torch thread pools): all threads on the whole
    stack (best of 3) and one thread on the first 8 frames"""
    threads = len(os.sched_getaffinity(0))

    def child(frames, thr, repeats):
        cmd = [sys.executable, os.path.abspath(__file__), '--cpu-child',
               '--frames', str(args.frames), '--seed', str(1000 + rank),
               '--cpu-frames', str(frames), '--cpu-threads', str(thr), '--repeats', str(repeats)]
        out = subprocess.run(cmd, capture_output=True, text=True, timeout=900, check=True)
        return json.loads(out.stdout.strip().splitlines()[-1])

    allc = child(args.cpu_frames, threads, 3)
    one = child(8, 1, 1)
    return {'value': allc['lines'] / allc['seconds'] / 1e6, 'unit': 'Mlines/s',
            'cores': threads, 'kind': 'port',
            'sample': f"{allc['frames']} of {args.frames} frames ({allc['lines']} lines), best "
                      "of 3, out zeroed and touched before the clock, fresh process",
            'cpu_model': cpu_model(),
            'one_thread': {'value': one['lines'] / one['seconds'] / 1e6, 'unit': 'Mlines/s',
                           'cores': 1,
                           'sample': f"{one['frames']} frames ({one['lines']} lines), one run"}}


def run_reference(args, ls, world, rank):
    if rank != 0:
        return
    import oracle  # noqa: F401  (builds the C port on first use)
    cfg = workload_config(ls)
    threads = len(os.sched_getaffinity(0))
    frames = args.cpu_frames
    for _ in range(max(args.warmup, 1)):
        probe = time_oracle(ls, 2, threads, 1)
    if frames <= 0:
        # about 60 s of CPU work over all timed steps, at least one frame per step
        per_frame = probe['seconds'] / 2
        frames = int(min(ls.shape[0], max(1, round(60.0 / max(args.steps, 1) / per_frame))))
    vals = [time_oracle(ls, frames, threads, 1) for _ in range(args.steps)]
    secs = sum(v['seconds'] for v in vals)
    lines = sum(v['lines'] for v in vals)
    value = lines / secs / 1e6
    cb = {'value': value, 'unit': 'Mlines/s', 'cores': threads, 'kind': 'port',
          'sample': f'the first {frames} of {ls.shape[0]} frames per step, out zeroed and '
                    'touched before the clock',
          'cpu_model': cpu_model()}
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


def measure_fit(steps: int, warmup: int, rank: int, local: int, fd_params: int = 32):
    """forward + loss + adjoint iterations on the 8 x 1024^2 workload, next to a
    finite-difference gradient from the plain forward: 2 forwards and a loss per
    parameter, 5 parameters per line.  The finite differences of `fd_params`
    parameters are run and timed (the whole stack per forward, and the parameter's own
    frame only), the full gradient's cost is that time scaled to 5 N parameters."""
    import torch
    from cbclib_v2_gb300 import autograd, draw_lines, fit, workloads
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

    def timed(fn, k):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(k):
            r = fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / k, r

    ms_iter, _ = timed(fused_step, steps)           # forward + fused loss adjoint
    ms_autograd, loss = timed(step, max(steps // 4, 3))   # torch autograd, torch loss
    out = torch.zeros(ls.shape, device='cuda')

    def forward():
        out.zero_()
        draw_lines(out, truth, idxs, ls.max_val, ls.kernel, ls.overlap)

    ms_fwd, _ = timed(forward, steps)
    # finite differences, really run: parameter j of line i moved by +-1e-3 px
    h = 1e-3
    rng = np.random.default_rng(11)
    sel = rng.choice(ls.n_lines * 5, size=fd_params, replace=False)
    p = truth.clone()
    fd = torch.empty(fd_params, dtype=torch.float64, device='cuda')
    offs = ls.frame_offsets()

    def loss_of(q):
        out.zero_()
        draw_lines(out, q, idxs, ls.max_val, ls.kernel, ls.overlap)
        return ((out - target) ** 2).sum(dtype=torch.float64)

    def fd_whole():
        for k, j in enumerate(sel):
            i, c = divmod(int(j), 5)
            p[i, c] += h
            lp = loss_of(p)
            p[i, c] -= 2 * h
            lm = loss_of(p)
            p[i, c] += h
            fd[k] = (lp - lm) / (2 * h)

    frame_out = torch.zeros(ls.shape[1:], device='cuda')

    def fd_frame():
        for k, j in enumerate(sel):
            i, c = divmod(int(j), 5)
            f = int(ls.idxs[i])
            q = p[offs[f]:offs[f + 1]]
            t = target[f]
            vals = []
            for sgn in (1, -1):
                p[i, c] += sgn * h
                frame_out.zero_()
                draw_lines(frame_out, q, None, ls.max_val, ls.kernel, ls.overlap)
                vals.append(((frame_out - t) ** 2).sum(dtype=torch.float64))
                p[i, c] -= sgn * h
            fd[k] = (vals[0] - vals[1]) / (2 * h)

    fd_whole()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fd_whole()
    torch.cuda.synchronize()
    ms_fd_whole = (time.perf_counter() - t0) * 1e3 / fd_params
    fd_frame()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fd_frame()
    torch.cuda.synchronize()
    ms_fd_frame = (time.perf_counter() - t0) * 1e3 / fd_params
    n_params = 5 * ls.n_lines
    return {
        'workload': ls.name, 'frames': ls.shape[0], 'lines': ls.n_lines,
        'kernel': ls.kernel, 'overlap': ls.overlap,
        'loss': 'sum((I - target)^2), target = Poisson(render(perturbed lines))',
        'metric': 'forward+adjoint iterations/s', 'value': 1e3 / ms_iter, 'unit': 'iter/s',
        'ms_per_iter': ms_iter, 'steps': steps,
        'path': 'fused: draw_lines + squared-loss adjoint (2 (I - T) per drawn pixel)',
        'autograd_ms_per_iter': ms_autograd, 'forward_ms': ms_fwd,
        'finite_difference': {
            'step_px': h, 'params_run': fd_params, 'params_total': n_params,
            'ms_per_param_whole_stack': ms_fd_whole,
            'ms_per_param_own_frame': ms_fd_frame,
            'gradient_ms_whole_stack': ms_fd_whole * n_params,
            'gradient_ms_own_frame': ms_fd_frame * n_params,
            'how': 'measured on the parameters run (2 forwards + a float64 loss each, '
                   'wall clock with the GPU synchronised), scaled to 5 N parameters'},
        'speedup_vs_finite_difference': ms_fd_whole * n_params / ms_iter,
        'speedup_vs_finite_difference_own_frame': ms_fd_frame * n_params / ms_iter,
        'loss_value': float(loss.item())}


def run_fit(args, world, rank, local):
    r = measure_fit(args.steps, args.warmup, rank, local)
    if rank == 0:
        print(json.dumps({
            'metric': 'forward+adjoint iterations/s', 'value': r['value'] * world,
            'unit': 'iter/s', 'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': r['ms_per_iter'], 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
            'config': {k: r[k] for k in ('workload', 'frames', 'lines', 'kernel', 'overlap',
                                         'loss')},
            **{k: r[k] for k in ('path', 'autograd_ms_per_iter', 'forward_ms',
                                 'finite_difference', 'speedup_vs_finite_difference',
                                 'speedup_vs_finite_difference_own_frame')}}), flush=True)


def measure_ragged(steps: int, warmup: int, rank: int, local: int, frames: int = 256):
    """256 frames of 1024^2, lognormal(median 1,500, sigma 1) segments per frame clipped
    to [100, 20,000], triangular, sum: one graph replay of the autotuned CSR draw per
    step, against one eager draw_lines_csr call of the same stack and one public
    draw_lines call per frame"""
    import torch
    from cbclib_v2_gb300 import batch, ndimage, workloads
    torch.cuda.set_device(local)
    ls = workloads.ragged_stack(seed=3000 + rank, F=frames)
    offs = ls.frame_offsets()
    lines = torch.from_numpy(ls.lines.astype(np.float32)).cuda()
    r = batch.RaggedRenderer(ls.shape, offs, max_val=ls.max_val, kernel=ls.kernel,
                             overlap=ls.overlap)
    r(lines)
    r.check()
    stream = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn, k):
        for _ in range(max(warmup, 1)):
            fn()
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(k):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / k

    ms_graph = timed(r.replay, steps)
    r.check()
    out = torch.zeros(ls.shape, device='cuda')
    d_offs = torch.from_numpy(offs).cuda()
    ms_eager = timed(lambda: ndimage.draw_lines_csr(out, lines, d_offs, ls.max_val, ls.kernel,
                                                    ls.overlap, tuning=r.tuning), steps)
    ms_frames = timed(lambda: batch.render_per_frame(out, lines, offs, ls.max_val, ls.kernel,
                                                     ls.overlap), max(2, steps // 10))
    t = r.tuning
    return {
        'workload': ls.name, 'frames': ls.shape[0], 'lines': ls.n_lines,
        'lines_per_frame_min_max': [int(np.diff(offs).min()), int(np.diff(offs).max())],
        'kernel': ls.kernel, 'overlap': ls.overlap,
        'metric': 'ragged draw_lines throughput', 'value': ls.n_lines / ms_graph / 1e3,
        'unit': 'Mlines/s', 'ms_graph_replay': ms_graph, 'steps': steps,
        'autotuned': {f: getattr(t, f) for f, _ in type(t)._fields_} if t is not None else None,
        'autotune_ms': r.timings,
        'ms_eager_csr_call': ms_eager, 'ms_per_frame_launches': ms_frames,
        'graph_speedup_vs_eager_csr_call': ms_eager / ms_graph,
        'graph_speedup_vs_per_frame': ms_frames / ms_graph}


def run_ragged(args, world, rank, local):
    r = measure_ragged(args.steps, args.warmup, rank, local,
                       args.frames if args.frames_given else 256)
    if rank == 0:
        print(json.dumps({
            'metric': r['metric'], 'value': world * r['value'], 'unit': 'Mlines/s',
            'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': r['ms_graph_replay'], 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
            'config': {k: r[k] for k in ('workload', 'frames', 'lines',
                                         'lines_per_frame_min_max', 'kernel', 'overlap')},
            **{k: r[k] for k in ('autotuned', 'autotune_ms', 'ms_eager_csr_call',
                                 'ms_per_frame_launches', 'graph_speedup_vs_eager_csr_call',
                                 'graph_speedup_vs_per_frame')}}), flush=True)


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
    adj3 = _draw3d_adjoint_times(ts, lines, terms, frames, dev) \
        if args.workload == 'rotomap' else None
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
            'clocks': clocks, 'gpu_launches': prof.launches, 'cpu_baseline': cb,
            'draw3d_adjoint': adj3}), flush=True)


def _draw3d_adjoint_times(ts, lines, terms, frames, dev):
    """the workload's 3-D lines drawn with draw_lines into their volumes, and the
    adjoint of that draw (gradient of sum(g * volumes) for a random g), sum and max
    overlap: ms per call, CUDA events over 20 calls after 3 warm-up calls"""
    import torch
    from cbclib_v2_gb300 import autograd, draw_lines
    idxs = frames.long()[terms.long()]
    vol = torch.zeros(ts.shape, dtype=torch.float32, device=dev)
    g = torch.rand(ts.shape, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def timed(fn, n=20):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(n):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / n

    res = {'kernel': ts.kernel, 'lines': ts.n_lines}
    for ov in ('sum', 'max'):
        vol.zero_()
        draw_lines(vol, lines, idxs, ts.max_val, ts.kernel, ov)
        image = vol.clone()
        res[ov] = {
            'forward_ms': timed(lambda: draw_lines(vol, lines, idxs, ts.max_val, ts.kernel, ov)),
            'adjoint_ms': timed(lambda: autograd.lines_backward(
                g, lines, idxs, ts.max_val, ts.kernel, ov, image=image if ov == 'max' else None))}
    return res


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


def measure_fit_loop(steps: int, warmup: int, rank: int, local: int, frames: int = 32,
                     split=None):
    """the streak-fit loop: 32 frames of 2167x2070, 5,000 biweight lines per frame,
    max overlap; the target is Poisson noise on the render of the true lines (peak 100
    counts), the start is the truth perturbed by N(0, 1 px) on the endpoints and
    N(0, 0.3 px) on the widths; `steps` Adam steps of lr 0.05; steps/s and the
    parameter RMS against the truth before and after.  `split` = (rank, world)
    fits only this rank's share of the frames (shard.partition_frames)."""
    import torch
    from cbclib_v2_gb300 import draw_lines, fit, workloads
    torch.cuda.set_device(local)
    ls = workloads.fit_loop_stack(seed=4000 + (0 if split else rank), F=frames)
    if split is not None:
        from cbclib_v2_gb300 import shard
        sh = shard.shard_of(ls.frame_offsets(), *split)
        ls = workloads.frames_subset(ls, list(range(sh.f0, sh.f1)))
    dev = torch.device('cuda', local)
    truth = torch.from_numpy(ls.lines.astype(np.float32)).to(dev)
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).to(dev)
    target = torch.zeros(ls.shape, device=dev)
    draw_lines(target, truth, idxs, ls.max_val, ls.kernel, ls.overlap)
    gen = torch.Generator(device=dev).manual_seed(4200 + rank)
    target = torch.poisson(target, generator=gen)          # counts, peak 100 per line
    start = torch.from_numpy(workloads.perturbed(ls.lines, 4100 + rank, 1.0, 0.3)
                             .astype(np.float32)).to(dev)
    fit.fit_lines(target, start, idxs, max_val=ls.max_val, kernel=ls.kernel,
                  overlap=ls.overlap, steps=max(warmup, 1), lr=0.05)      # warm-up
    res = fit.fit_lines(target, start, idxs, max_val=ls.max_val, kernel=ls.kernel,
                        overlap=ls.overlap, steps=steps, lr=0.05)

    def rms(p):
        d = (p - truth).double()
        return {'endpoints_px': float(d[:, :4].pow(2).mean().sqrt()),
                'width_px': float(d[:, 4].pow(2).mean().sqrt())}

    return {
        'workload': ls.name, 'frames': ls.shape[0], 'lines': ls.n_lines,
        'kernel': ls.kernel, 'overlap': ls.overlap, 'lr': 0.05,
        'loss': 'sum((I - T)^2), T = Poisson(render of the true lines), peak 100 counts',
        'start': 'truth + N(0, 1 px) endpoints, N(0, 0.3 px) widths',
        'metric': 'streak-fit Adam steps/s', 'value': 1e3 / res.ms_per_step,
        'unit': 'steps/s', 'ms_per_step': res.ms_per_step, 'steps': steps,
        'rms_start': rms(start), 'rms_final': rms(res.lines),
        'loss_start': res.losses[0], 'loss_final': res.losses[-1]}


def run_fit_loop(args, world, rank, local):
    frames = args.frames if args.frames_given else 32
    steps = args.steps if args.steps_given else 100
    split = (rank, world) if (args.shard and world > 1) else None
    r = measure_fit_loop(steps, args.warmup, rank, local, frames, split)
    if rank == 0:
        print(json.dumps({
            'metric': r['metric'], 'value': (world if split is None else 1) * r['value'],
            'unit': 'steps/s', 'n_gpus': world, 'steps': steps, 'warmup': args.warmup,
            'ms_per_step': r['ms_per_step'], 'higher_is_better': True,
            'scaling': 'strong' if split else 'weak', 'vs_baseline': None, 'dtype': 'f32',
            'data': 'synthetic',
            'config': {k: r[k] for k in ('workload', 'frames', 'lines', 'kernel', 'overlap',
                                         'lr', 'loss', 'start')},
            **{k: r[k] for k in ('rms_start', 'rms_final', 'loss_start', 'loss_final')}}),
            flush=True)


def e2e_step_bytes(n_lines: int, drawn: int):
    """bytes across the link per step: lines (5 float32) and int32 indices up, the
    drawn pixels read and written in place in the host frames"""
    return {'h2d_bytes_per_step': int(n_lines * 20 + n_lines * 4 + drawn * 4),
            'd2h_bytes_per_step': int(drawn * 4)}


def main():
    args = parse()
    if args.cpu_child:
        cpu_child(args)
        return
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
    from cbclib_v2_gb300 import workloads

    split = args.shard and world > 1
    ls = workloads.detector_stack(seed=1000 + (0 if split else rank), F=args.frames)
    if args.impl == 'reference':
        run_reference(args, ls, world, rank)
        return
    import torch
    from cbclib_v2_gb300 import _native, draw_lines, ndimage, shard

    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl', init_method='env://')
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    full_lines = ls.n_lines
    if split:
        # this rank's contiguous frame range of the one stack, balanced by line counts
        sh = shard.shard_of(ls.frame_offsets(), rank, world)
        ls = workloads.frames_subset(ls, list(range(sh.f0, sh.f1)))
    F, H, W = ls.shape
    N = ls.n_lines
    lines = torch.from_numpy(ls.lines.astype(np.float32)).to(dev)
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).to(dev)
    out = torch.zeros(ls.shape, dtype=torch.float32, device=dev)

    def barrier():
        if dist is not None:
            dist.barrier(device_ids=[local])

    def max_over_ranks(ms):
        if dist is None:
            return ms
        tt = torch.tensor([ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        return float(tt.item())

    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(args.warmup):
        draw_lines(out, lines, idxs, ls.max_val, ls.kernel, ls.overlap)
    torch.cuda.synchronize()
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
    ms_step = max_over_ranks(t0.elapsed_time(t1)) / args.steps
    total_lines = full_lines if split else world * N
    value = total_lines / (ms_step * 1e-3) / 1e6

    # the same calls inside ndimage.deferred_errors(): the status of each call is
    # checked once after the last instead of after each, so calls queue back to back
    with ndimage.deferred_errors():
        for _ in range(max(args.warmup, 1)):
            draw_lines(out, lines, idxs, ls.max_val, ls.kernel, ls.overlap)
    barrier()
    torch.cuda.synchronize()
    d0, d1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ndimage.deferred_errors():
        d0.record(stream)
        for _ in range(args.steps):
            draw_lines(out, lines, idxs, ls.max_val, ls.kernel, ls.overlap)
        d1.record(stream)
    torch.cuda.synchronize()
    ms_deferred = max_over_ranks(d0.elapsed_time(d1)) / args.steps

    # the drawn pixels (the bytes that cross the link in place, and the sparse model)
    ref = torch.zeros(ls.shape, dtype=torch.float32, device=dev)
    draw_lines(ref, lines, idxs, ls.max_val, ls.kernel, ls.overlap)
    drawn = int((ref != 0).sum())
    drawn_sectors = int(ref.reshape(-1, 8).ne(0).any(dim=1).sum().item())
    del ref

    def e2e_run(h_out, h_lines, h_idxs, what):
        for _ in range(max(1, args.warmup)):
            draw_lines(h_out, h_lines, h_idxs, ls.max_val, ls.kernel, ls.overlap)
        e_steps = max(3, min(args.steps // 4, 50))
        barrier()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        w0 = time.perf_counter()
        a.record(stream)
        for _ in range(e_steps):
            draw_lines(h_out, h_lines, h_idxs, ls.max_val, ls.kernel, ls.overlap)
        b.record(stream)
        torch.cuda.synchronize()
        wall = (time.perf_counter() - w0) * 1e3 / e_steps
        barrier()
        e_ms = max_over_ranks(a.elapsed_time(b) / e_steps)
        return {'value': total_lines / (e_ms * 1e-3) / 1e6, 'unit': 'Mlines/s',
                'ms_per_step': e_ms, 'wall_ms_per_step': wall, 'steps': e_steps,
                **e2e_step_bytes(N, drawn),
                'frames': what + '; %d of %d pixels drawn' % (drawn, F * H * W)}

    # end to end through the public API with host buffers: NumPy arrays (what the
    # reference's callers pass), then page-locked torch tensors
    e2e = e2e_pinned = None
    if not args.no_e2e:
        n_out = np.zeros(ls.shape, np.float32)
        n_out.fill(0.0)
        n_lines = np.ascontiguousarray(ls.lines.astype(np.float32))
        n_idxs = np.ascontiguousarray(ls.idxs.astype(np.int32))
        mode = _native.host_access(n_out.ctypes.data)
        e2e = e2e_run(n_out, n_lines, n_idxs,
                      'NumPy arrays in pageable host memory, drawn pixels combined in place '
                      'by the kernels (zero-copy over NVLink-C2C)' if mode == _native.HOST_PAGEABLE
                      else 'NumPy arrays, copied to the device and back')
        del n_out
        h_out = torch.zeros(ls.shape, dtype=torch.float32).pin_memory()
        h_lines = torch.from_numpy(ls.lines.astype(np.float32)).pin_memory()
        h_idxs = torch.from_numpy(ls.idxs.astype(np.int32)).pin_memory()
        e2e_pinned = e2e_run(h_out, h_lines, h_idxs,
                             'page-locked torch tensors, drawn pixels combined in place by '
                             'the kernels (zero-copy)')
        del h_out

    extra = {}
    if not args.headline_only:
        steps_x = max(args.steps, 20)
        extra['forward_adjoint'] = measure_fit(min(steps_x, 200), max(args.warmup, 3), rank, local)
        extra['ragged_graph'] = measure_ragged(min(steps_x, 100), max(args.warmup, 3), rank,
                                               local)
        extra['fit_loop'] = measure_fit_loop(100, max(args.warmup, 3), rank, local)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    peak, peak_src = measured_peak()
    render_ms = prof.ms_render / max(prof.calls, 1)
    kname = 'segments_kernel' if strategy == _native.STRATEGY_LINES else 'render_kernel'
    # bytes the op must move: the in-place contract reads and writes every output pixel
    # once, plus each line's 5 coordinates and frame index; the sparse model counts the
    # 32-byte sectors holding a drawn pixel (all other sectors are untouched)
    algo_bytes = 64 * drawn_sectors + N * 24
    full_bytes = 2 * F * H * W * 4 + N * 24
    achieved = full_bytes / (render_ms * 1e-3) / 1e9
    sparse = algo_bytes / (render_ms * 1e-3) / 1e9
    traffic = committed_traffic(ls.name, kname) if not split else None
    roofline = {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                'frac': achieved / peak, 'peak_source': peak_src,
                'traffic': traffic, 'kernel': kname,
                'traffic_frac': (traffic / (render_ms * 1e-3) / 1e9 / peak) if traffic else None,
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
    cfg = workload_config(ls)
    if split:
        cfg['sharding'] = f'one {args.frames}-frame stack split by frames across {world} ranks'
    res = {
        'metric': 'draw_lines throughput', 'value': value, 'unit': 'Mlines/s', 'n_gpus': world,
        'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms_step,
        'higher_is_better': True, 'scaling': 'strong' if split else 'weak', 'vs_baseline': None,
        'dtype': 'f32', 'data': 'synthetic', 'config': cfg, 'roofline': roofline,
        'output_gbs': F * H * W * 4 / (ms_step * 1e-3) / 1e9, 'clocks': clk,
        'gpu_launches': prof.launches, 'e2e': e2e, 'e2e_pinned': e2e_pinned,
        'deferred_errors': {'value': total_lines / (ms_deferred * 1e-3) / 1e6,
                            'unit': 'Mlines/s', 'ms_per_step': ms_deferred,
                            'how': 'the same calls inside ndimage.deferred_errors(): device '
                                   'status checked once after the last call'},
    }
    if extra:
        res['workloads'] = extra
    if not args.no_cpu_baseline and world == 1:
        res['cpu_baseline'] = cpu_baseline(args, rank)
    print(json.dumps(res), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
