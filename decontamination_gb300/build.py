"""Builds libsomgb.so (the CUDA kernels and their C ABI) in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into
``decontamination_gb300/libsomgb.so`` next to this file. ``python -m
decontamination_gb300.build`` runs it; ``__graft_entry__.build()`` calls
``build()``.
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
LIB = os.path.join(HERE, 'libsomgb.so')
OBJ_DIR = os.path.join(HERE, '_build')

SOURCES = ['api.cu', 'k0_fp32.cu', 'k1_tc.cu', 'k_update.cu', 'k_moments.cu', 'k_sort.cu', 'k4_iter_tc.cu', 'noalloc.cu']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-Wall',
              '--expt-relaxed-constexpr']


def nvcc():
    cand = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(cand):
        raise RuntimeError('nvcc not found; the CUDA toolkit is required to build libsomgb.so')
    return cand


def _compile(src, verbose):
    obj = os.path.join(OBJ_DIR, os.path.splitext(src)[0] + '.o')
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, '-c', os.path.join(CSRC, src), '-o', obj]
    if verbose:
        cmd.insert(1, '-Xptxas=-v')
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f'nvcc failed on {src}:\n{res.stdout}\n{res.stderr}')
    return obj, res.stderr


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, '..', 'include', 'somgb.h'),
                                                               __file__]
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def build(force=False, verbose=False):
    """Compile and link libsomgb.so if any source is newer than it. Returns the library path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + '.tmp'
    cmd = [nvcc(), *ARCH, '-shared', '--cudart', 'static', '-o', tmp, *objs]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f'link failed:\n{res.stdout}\n{res.stderr}')
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
