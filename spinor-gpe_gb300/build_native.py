"""Build the CUDA library ``libspinor_gb300.so`` in-tree for sm_103a.

Usage: ``python spinor-gpe_gb300/build_native.py`` (or ``build()`` from
Python).  Each translation unit in ``csrc/`` is compiled by its own nvcc
process in parallel, then linked into
``spinor-gpe_gb300/spinor_gpe/libspinor_gb300.so``, where the Python package
loads it from.  Objects go to ``spinor-gpe_gb300/_build/``.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, 'csrc')
INCLUDE = os.path.join(REPO, 'include')
BUILD = os.path.join(PKG_ROOT, '_build')
LIB = os.path.join(PKG_ROOT, 'spinor_gpe', 'libspinor_gb300.so')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC',
         '-I' + INCLUDE, '-I' + CSRC]


def _nvcc():
    exe = shutil.which('nvcc')
    if exe is None:
        cand = '/usr/local/cuda/bin/nvcc'
        if os.path.exists(cand):
            exe = cand
    if exe is None:
        raise RuntimeError('nvcc not found: the CUDA toolkit is required to '
                           'build libspinor_gb300.so')
    return exe


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith('.cu'))


def _stale(lib, deps):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=(), lib_path=None,
          build_dir=None, reuse_objects=()):
    """Compile and link the library; returns its path.  Skips the work when
    the library is newer than every source and header.  ``lib_path`` /
    ``build_dir`` redirect the outputs (tuning builds); object files named in
    ``reuse_objects`` (basenames without .o) are linked from ``build_dir``
    as they are instead of being recompiled."""
    lib = lib_path or LIB
    bdir = build_dir or BUILD
    srcs = _sources()
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC)
                   if f.endswith('.cuh')]
    deps.append(os.path.join(INCLUDE, 'spinor_gb300.h'))
    if not force and not extra_flags and not _stale(lib, deps):
        return lib
    os.makedirs(bdir, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        name = os.path.basename(src)[:-3]
        obj = os.path.join(bdir, name + '.o')
        if name in reuse_objects and os.path.exists(obj):
            return obj
        cmd = [nvcc, *ARCH, *FLAGS, *extra_flags, '-c', src, '-o', obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f'nvcc failed for {src}:\n{res.stderr}')
        if verbose:
            sys.stderr.write(res.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib + '.tmp'
    cmd = [nvcc, *ARCH, '-shared', '-o', tmp, *objs]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f'link failed:\n{res.stderr}')
    os.replace(tmp, lib)
    return lib


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
