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
