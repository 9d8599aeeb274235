"""Build libpynufft_gb300.so in-tree for sm_103a.

    python -m pynufft_gb300.build          # or: from pynufft_gb300.build import build

Each CUDA/C++ translation unit is compiled by nvcc in parallel into
``pynufft_gb300/_build/`` and linked with cuFFT into
``pynufft_gb300/libpynufft_gb300.so``.  Only the sm_103a target is generated.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libpynufft_gb300.so')
SOURCES = ['capi.cu', 'plan_math.cpp', 'points.cu', 'interp.cu', 'interp_d1.cu', 'interp_d2.cu',
           'interp_d3.cu', 'interp_cm2.cu', 'interp_cm3.cu', 'fftstage.cu', 'pfft.cu', 'cfft.cu', 'cg.cu', 'tv.cu', 'noalloc.cu', 'selftest.cu']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def _cuda_home() -> str:
    for c in (os.environ.get('CUDA_HOME'), os.environ.get('CUDA_PATH'), '/usr/local/cuda'):
        if c and os.path.exists(os.path.join(c, 'bin', 'nvcc')):
            return c
    nvcc = shutil.which('nvcc')
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError('nvcc not found; set CUDA_HOME')


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_verbose: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, 'bin', 'nvcc')
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.cuh', '.h'))]
    headers.append(os.path.join(HERE, '..', 'include', 'pynufft_gb300.h'))
    sources = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    common = ['-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr']
    if ptxas_verbose:
        common += ['-Xptxas', '-v']
    jobs = []
    for src in sources:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + '.o')
        if force or _stale(obj, [path] + headers + [__file__]):
            cmd = [nvcc] + ARCH + common + ['-c', path, '-o', obj]
            if src.endswith('.cpp'):
                cmd = [nvcc] + common + ['-x', 'c++', '-c', path, '-o', obj]
            jobs.append((src, cmd))

    def run(job):
        src, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, r

    failed = []
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for src, r in ex.map(run, jobs):
            if verbose or r.returncode != 0 or ptxas_verbose:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                failed.append(src)
    if failed:
        raise RuntimeError('nvcc failed for: ' + ', '.join(failed))
    objs = [os.path.join(BUILD, s + '.o') for s in sources]
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + '.tmp'
        cmd = [nvcc] + ARCH + ['-shared', '-cudart', 'shared', '-o', tmp] + objs + \
              ['-L' + os.path.join(cuda, 'lib64'), '-lcufft',
               '-Xlinker', '-rpath,' + os.path.join(cuda, 'lib64')]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError('link failed')
        os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    build(verbose='-v' in sys.argv, force='-f' in sys.argv, ptxas_verbose='--ptxas' in sys.argv)
    print(LIB)
