"""ORACLE — test infrastructure only.  The reference project's own GPU module
``cuda_draw_lines`` (cbclib_v2/_src/src/cuda_draw_lines.cu), compiled unmodified for
sm_103a by ``oracle/build_ref_cuda.sh`` from sources staged into ``oracle/_ref/cuda_src``
(git-ignored).  Used to time the reference's GPU path beside this library and to
compare outputs; never imported by the package.

``module(build=True)`` returns the module, compiling it first when the staged sources
exist and no build is present, or None.  Its ``draw_lines(out, lines, idxs, max_val,
kernel, overlap)`` takes any ``__cuda_array_interface__`` arrays (torch CUDA tensors):
float32 frames with int32 indices, or float64 with int64 (its pybind11 overloads,
cuda_draw_lines.cu:1098-1113)."""
import glob
import importlib.util
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, '_ref')
_mod = None


def staged() -> bool:
    return os.path.exists(os.path.join(REF, 'cuda_src', 'cuda_draw_lines.cu'))


def build() -> str:
    out = subprocess.run(['bash', os.path.join(HERE, 'build_ref_cuda.sh'), 'build'],
                         capture_output=True, text=True, timeout=1200)
    if out.returncode != 0:
        raise RuntimeError('building the reference CUDA module failed:\n' + out.stderr[-3000:])
    return out.stdout.strip().splitlines()[-1]


def module(build_if_missing: bool = True):
    global _mod
    if _mod is not None:
        return _mod
    import sysconfig
    path = os.path.join(REF, 'cuda_draw_lines' + sysconfig.get_config_var('EXT_SUFFIX'))
    if not os.path.exists(path):
        if not (build_if_missing and staged()):
            return None
        path = build()
    spec = importlib.util.spec_from_file_location('cuda_draw_lines', path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    _mod = mod
    return mod


def compare_detector_stack(frames: int = 64, steps: int = 5) -> dict:
    """The reference GPU module and this library on the detector-stack workload (64
    frames of 2167x2070, Poisson(2,000) segments per frame, int32 frame indices,
    max overlap): wall time per call with the GPU synchronised before and after (the
    reference's call synchronises inside), best and median of `steps` calls into
    zeroed frames, for the gaussian and the rectangular profile, and the pixels on
    which the two results differ."""
    import time
    import numpy as np
    import torch
    from cbclib_v2_gb300 import draw_lines, workloads
    mod = module()
    if mod is None:
        raise RuntimeError("reference CUDA module unavailable (oracle/build_ref_cuda.sh stage)")
    ls = workloads.detector_stack(seed=1000, F=frames)
    lines = torch.from_numpy(ls.lines.astype(np.float32)).cuda()
    idxs = torch.from_numpy(ls.idxs.astype(np.int32)).cuda()

    def timed(fn, out, k):
        fn(out)
        ts = []
        for _ in range(k):
            out.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn(out)
            torch.cuda.synchronize()
            ts.append((time.perf_counter() - t0) * 1e3)
        return min(ts), sorted(ts)[len(ts) // 2]

    res = {'workload': ls.name, 'lines': ls.n_lines, 'overlap': 'max'}
    for kernel in ('gaussian', 'rectangular'):
        ref = torch.zeros(ls.shape, device='cuda')
        ours = torch.zeros(ls.shape, device='cuda')
        r_best, r_med = timed(lambda o: mod.draw_lines(o, lines, idxs, 1.0, kernel, 'max'), ref,
                              steps)
        o_best, o_med = timed(lambda o: draw_lines(o, lines, idxs, 1.0, kernel, 'max'), ours,
                              4 * steps)
        res[kernel] = {'reference_ms_best': r_best, 'reference_ms_median': r_med,
                       'this_library_ms_best': o_best, 'this_library_ms_median': o_med,
                       'speedup_median': r_med / o_med,
                       'pixels_differing': int((ref != ours).sum()),
                       'pixels_drawn': int((ours != 0).sum()),
                       'max_abs_difference': float((ref - ours).abs().max())}
    return res


if __name__ == '__main__':
    import json
    import sys
    sys.path.insert(0, os.path.dirname(HERE))
    print(json.dumps(compare_detector_stack()))
