"""Builds libvissat_gb300.so (sm_103a) in-tree with nvcc.

    python -m vissatsatellitestereo_gb300.build [--force]

Each CUDA translation unit under csrc/ is compiled in parallel into _build/, then linked
into the package directory.  Objects are rebuilt only when a source or header is newer.
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, 'csrc')
BUILD = os.path.join(PKG, '_build')
LIB = os.path.join(PKG, 'libvissat_gb300.so')
INCLUDE = os.path.join(os.path.dirname(PKG), 'include')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-O2',
              '--expt-relaxed-constexpr']


def nvcc():
    path = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(path):
        raise RuntimeError('nvcc not found: the CUDA toolkit is required to build vissat-gb300')
    return path


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith('.cu'))


def _deps_mtime():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.cuh', '.h'))]
    hdrs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith('.h')]
    return max(os.path.getmtime(h) for h in hdrs)


def _compile(src, force):
    obj = os.path.join(BUILD, src[:-3] + '.o')
    srcp = os.path.join(CSRC, src)
    if not force and os.path.exists(obj):
        if os.path.getmtime(obj) >= max(os.path.getmtime(srcp), _deps_mtime()):
            return obj, None
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ['-I', INCLUDE, '-c', srcp, '-o', obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        return obj, f'{" ".join(cmd)}\n{p.stdout}\n{p.stderr}'
    return obj, None


def build(force=False, verbose=False):
    """Compile every CUDA source for sm_103a and link the shared library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, force), srcs))
    errors = [e for _, e in results if e]
    if errors:
        raise RuntimeError('CUDA build failed:\n' + '\n'.join(errors))
    objs = [o for o, _ in results]
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + '.tmp'
        cmd = [nvcc()] + ARCH + ['-shared', '-o', tmp] + objs
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f'link failed:\n{" ".join(cmd)}\n{p.stdout}\n{p.stderr}')
        os.replace(tmp, LIB)
    if verbose:
        print('built', LIB)
    return LIB


if __name__ == '__main__':
    ap = argparse.ArgumentParser()
    ap.add_argument('--force', action='store_true')
    a = ap.parse_args()
    try:
        build(force=a.force, verbose=True)
    except RuntimeError as e:
        print(e, file=sys.stderr)
        sys.exit(1)
