"""Build libbx.so (the C-ABI step library) in-tree with nvcc for sm_103a.

Each ``csrc/*.cu`` translation unit compiles in parallel to an object file;
the objects link into ``betse_gb300/libbx.so`` with the CUDA runtime linked
statically, so the library loads with no CUDA library path set.  Rebuilds only
when a source or header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libbx.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-O2',
         '--expt-relaxed-constexpr', '-Xptxas', '-warn-spills']


def nvcc() -> str:
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: the CUDA toolkit is required to build libbx.so')


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, '*.cu')))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, '*.cuh')) + \
        glob.glob(os.path.join(ROOT, 'include', '*.h')) + [os.path.abspath(__file__)]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    incs = ['-I' + os.path.join(ROOT, 'include'), '-I' + CSRC]

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src).replace('.cu', '.o'))
        cmd = [nv, *ARCH, *FLAGS, *extra_flags, *incs, '-c', src, '-o', obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f'nvcc failed for {src}:\n{r.stderr}')
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + '.tmp'
    cmd = [nv, *ARCH, '-shared', '-cudart', 'static', '-o', tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f'link failed:\n{r.stderr}')
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    import time
    t0 = time.time()
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv), f'{time.time() - t0:.1f} s')
