"""Build the C/OpenMP oracle (test infrastructure and CPU baseline).

Two shared libraries are produced in oracle/_build/:
  libfroracle_strict.so  -O3 -fopenmp, IEEE arithmetic (the checker)
  libfroracle_fast.so    -O3 -fopenmp -ffast-math, the compiler flags the
                         reference's OpenMP backend uses for its kernels
                         (pyfr/backends/openmp/compiler.py:76-96), minus
                         -march=native so the build is portable
"""

from pathlib import Path
import subprocess

HERE = Path(__file__).resolve().parent
OUT = HERE / '_build'

VARIANTS = {
    'strict': ['-O3', '-fopenmp'],
    'fast': ['-O3', '-fopenmp', '-ffast-math'],
}


def libpath(variant='strict'):
    return OUT / f'libfroracle_{variant}.so'


def build(force=False):
    OUT.mkdir(exist_ok=True)
    src = HERE / 'fr_oracle.c'
    for v, flags in VARIANTS.items():
        lib = libpath(v)
        if force or not lib.exists() or lib.stat().st_mtime < src.stat().st_mtime:
            cmd = ['gcc', '-std=c11', '-shared', '-fPIC', *flags, str(src),
                   '-o', str(lib), '-lm']
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode:
                raise RuntimeError(f'oracle build failed:\n{r.stderr}')
    return OUT


if __name__ == '__main__':
    print(build(force=True))
