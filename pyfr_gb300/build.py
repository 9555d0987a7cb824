"""Build the pyfrb200 CUDA library in-tree for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled in parallel with nvcc and
linked into ``pyfr_gb300/_lib/libpyfrb200.so``; a unit is recompiled only
when it or a header is newer than its object file.
"""

from concurrent.futures import ThreadPoolExecutor
import os
from pathlib import Path
import shutil
import subprocess

PKG = Path(__file__).resolve().parent
CSRC = PKG / 'csrc'
LIBDIR = PKG / '_lib'
INCLUDE = PKG.parent / 'include'
LIBNAME = 'libpyfrb200.so'

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC',
              '--expt-relaxed-constexpr', '-I', str(INCLUDE)]


def nvcc_path():
    nvcc = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(nvcc):
        raise RuntimeError('nvcc not found')
    return nvcc


def _newest_header():
    hdrs = list(CSRC.glob('*.cuh')) + list(INCLUDE.glob('*.h'))
    return max((h.stat().st_mtime for h in hdrs), default=0)


def _compile(src, obj, verbose):
    cmd = [nvcc_path(), *ARCH, *NVCC_FLAGS, '-c', str(src), '-o', str(obj)]
    if verbose:
        cmd.insert(1, '-Xptxas=-v')
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f'nvcc failed for {src.name}:\n{r.stderr}')
    return r.stderr


def build(force=False, verbose=False, jobs=None):
    """Compile and link the library; returns its path."""
    LIBDIR.mkdir(exist_ok=True)
    objdir = LIBDIR / 'obj'
    objdir.mkdir(exist_ok=True)
    lib = LIBDIR / LIBNAME

    srcs = sorted(CSRC.glob('*.cu'))
    hdr_t = _newest_header()
    todo = []
    for s in srcs:
        o = objdir / (s.stem + '.o')
        if (force or not o.exists() or o.stat().st_mtime < s.stat().st_mtime
                or o.stat().st_mtime < hdr_t):
            todo.append((s, o))

    logs = []
    if todo:
        with ThreadPoolExecutor(jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(lambda so: _compile(*so, verbose), todo))

    objs = [objdir / (s.stem + '.o') for s in srcs]
    if todo or not lib.exists():
        tmp = lib.with_suffix('.so.tmp')
        cmd = [nvcc_path(), *ARCH, '-shared', '-o', str(tmp), *map(str, objs),
               '-lcudart']
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f'link failed:\n{r.stderr}')
        os.replace(tmp, lib)

    if verbose:
        for l in logs:
            print(l)

    return lib


if __name__ == '__main__':
    import sys
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
