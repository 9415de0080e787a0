"""Build the native library libcbc_gb300.so (CUDA kernels + C ABI) in-tree with nvcc
for sm_103a.  The output lands in cbclib_v2_gb300/_lib/ (git-ignored)."""
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, 'csrc')
INCLUDE = os.path.join(ROOT, 'include')
LIBDIR = os.path.join(PKG, '_lib')
LIB = os.path.join(LIBDIR, 'libcbc_gb300.so')
SOURCES = ['cbc_draw_lines.cu', 'cbc_adjoint.cu', 'cbc_accumulate.cu', 'cbc_lines3d.cu']
DEPS = ['exact.cuh', 'exp_table.inc', 'cbc_common.cuh', 'cbc_accumulate.cuh']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def nvcc() -> str:
    cand = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(cand):
        raise RuntimeError('nvcc not found: the CUDA 13 toolkit is required to build')
    return cand


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    files = [os.path.join(CSRC, f) for f in SOURCES + DEPS]
    files.append(os.path.join(INCLUDE, 'cbc_draw_lines.h'))
    files.append(os.path.abspath(__file__))
    return any(os.path.getmtime(f) > t for f in files)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    tmp = LIB + '.tmp'
    flags = [*ARCH, '-O3', '-lineinfo', '-std=c++17', '--fmad=false',
             '-Xcompiler', '-fPIC,-fvisibility=hidden', '-I', INCLUDE, '-I', CSRC]
    if verbose:
        flags += ['-Xptxas', '-v']
    objs = []
    procs = []
    for f in SOURCES:                       # translation units compile in parallel
        obj = os.path.join(LIBDIR, os.path.splitext(f)[0] + '.o')
        objs.append(obj)
        procs.append(subprocess.Popen([nvcc(), *flags, '-c', os.path.join(CSRC, f), '-o', obj]))
    if any(p.wait() != 0 for p in procs):
        raise RuntimeError('nvcc failed')
    subprocess.run([nvcc(), *ARCH, '-shared', '-o', tmp, *objs], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
