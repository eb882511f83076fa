"""Builds libdiffvg_gb300.so (the sm_103a kernels and the C ABI) and
libdvg_torch.so (PyTorch operators over the C ABI) in-tree.

nvcc compiles each translation unit of csrc/ in parallel and links them
into diffvg_gb300/_lib/libdiffvg_gb300.so; g++ compiles csrc/dvg_torch.cpp
against the installed PyTorch's headers (in parallel with the CUDA units)
and links it against that library.  No GPU is needed to build.
--fmad=false keeps every fp32 expression unfused so that sample
classification matches the reference's CPU arithmetic.
"""
import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
LIB_DIR = os.path.join(HERE, '_lib')
LIB_PATH = os.path.join(LIB_DIR, 'libdiffvg_gb300.so')
TORCH_LIB_PATH = os.path.join(LIB_DIR, 'libdvg_torch.so')
TORCH_UNIT = 'dvg_torch.cpp'
INCLUDE = os.path.join(os.path.dirname(HERE), 'include')

UNITS = ['dvg_prep.cu', 'dvg_render.cu', 'dvg_capi.cu', 'dvg_static.cu', 'dvg_optim.cu']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-std=c++17', '-lineinfo', '--fmad=false', '-Xcompiler', '-fPIC', '-Xcompiler', '-O2',
         '-I' + INCLUDE]


def _nvcc():
    cuda = os.environ.get('CUDA_HOME', '/usr/local/cuda')
    path = os.path.join(cuda, 'bin', 'nvcc')
    return path if os.path.exists(path) else (shutil.which('nvcc') or 'nvcc')


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.cu', '.cuh', '.h', '.cpp'))] + \
           [os.path.join(INCLUDE, 'diffvg_gb300.h')]


def up_to_date():
    if not (os.path.exists(LIB_PATH) and os.path.exists(TORCH_LIB_PATH)):
        return False
    t = min(os.path.getmtime(LIB_PATH), os.path.getmtime(TORCH_LIB_PATH))
    return all(os.path.getmtime(p) <= t for p in _sources() + [os.path.abspath(__file__)])


def _torch_flags():
    import torch
    tdir = os.path.dirname(os.path.abspath(torch.__file__))
    cuda = os.environ.get('CUDA_HOME', '/usr/local/cuda')
    inc = ['-I' + os.path.join(tdir, 'include'), '-I' + os.path.join(cuda, 'include'), '-I' + INCLUDE]
    abi = '-D_GLIBCXX_USE_CXX11_ABI=%d' % int(torch._C._GLIBCXX_USE_CXX11_ABI)
    tlib = os.path.join(tdir, 'lib')
    link = ['-L' + tlib, '-Wl,-rpath,' + tlib, '-lc10', '-lc10_cuda', '-ltorch_cpu',
            '-L' + LIB_DIR, '-Wl,-rpath,$ORIGIN', '-ldiffvg_gb300']
    return ['-O2', '-std=c++17', '-fPIC', abi] + inc, link


def build(force=False, verbose=False, extra_flags=()):
    """Compiles the library if a source changed; returns its path."""
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(LIB_DIR, exist_ok=True)
    nvcc = _nvcc()
    objs = []

    def compile_one(unit):
        src = os.path.join(CSRC, unit)
        obj = os.path.join(LIB_DIR, unit.replace('.cu', '.o'))
        cmd = [nvcc] + ARCH + FLAGS + list(extra_flags) + ['-c', src, '-o', obj]
        if verbose:
            print(' '.join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed on %s:\n%s%s' % (unit, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    cflags, lflags = _torch_flags()
    torch_obj = os.path.join(LIB_DIR, TORCH_UNIT.replace('.cpp', '.o'))

    def compile_torch():
        cmd = ['g++'] + cflags + ['-c', os.path.join(CSRC, TORCH_UNIT), '-o', torch_obj]
        if verbose:
            print(' '.join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('g++ failed on %s:\n%s%s' % (TORCH_UNIT, r.stdout, r.stderr))
        return torch_obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(UNITS) + 1) as ex:
        tjob = ex.submit(compile_torch)
        objs = list(ex.map(compile_one, UNITS))
        tjob.result()
    tmp = LIB_PATH + '.%d.tmp' % os.getpid()
    cmd = [nvcc] + ARCH + ['-shared', '-o', tmp] + objs + ['-lcudart']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('nvcc link failed:\n%s%s' % (r.stdout, r.stderr))
    os.replace(tmp, LIB_PATH)
    tmp = TORCH_LIB_PATH + '.%d.tmp' % os.getpid()
    cmd = ['g++', '-shared', '-o', tmp, torch_obj] + lflags
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('g++ link failed on %s:\n%s%s' % (TORCH_UNIT, r.stdout, r.stderr))
    os.replace(tmp, TORCH_LIB_PATH)
    return LIB_PATH


if __name__ == '__main__':
    import sys
    print(build(force='--force' in sys.argv, verbose=True,
                extra_flags=['-Xptxas', '-v'] if '--ptxas' in sys.argv else []))
