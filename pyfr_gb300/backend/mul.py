"""The ``mul`` kernel provider: out = alpha*A@B + beta*out.

Same contract as the reference's GiMMiK/cuBLASLt providers
(``pyfr/backends/cuda/gimmik.py:23-38``): A must be a constant matrix, a
shape mismatch raises ValueError.  The operator's nonzeros are uploaded
once per (matrix, device) and shared by every kernel that applies it.
"""

import ctypes as C

import numpy as np

from pyfr_gb300.backend.types import Kernel


class MulKernels:
    def __init__(self, backend):
        self.backend = backend
        self._handles = {}

    def _handle(self, a):
        key = a.mid
        if key not in self._handles:
            host = np.ascontiguousarray(a._host, dtype=np.float64)
            h = C.c_void_p()
            self.backend.lib.mul_create(
                host.ctypes.data_as(C.POINTER(C.c_double)), host.shape[0],
                host.shape[1], C.byref(h))
            nnz = C.c_int()
            self.backend.lib.mul_nnz(h, C.byref(nnz))
            self._handles[key] = (h.value, nnz.value, host)
        return self._handles[key]

    def mul(self, a, b, out, alpha=1.0, beta=0.0):
        if a.ncol != b.nrow or a.nrow != out.nrow or b.ncol != out.ncol:
            raise ValueError('Incompatible matrices for out = a*b')
        if 'const' not in a.tags:
            raise ValueError('The operator of mul must be a constant matrix')

        be = self.backend
        h, nnz, host = self._handle(a)
        ncol = b.ncol
        ldb, ldc = b.leaddim, out.leaddim

        if be.fpdtype == np.float64:
            fn, cv = be.lib.mul_f64, C.c_double
        else:
            fn, cv = be.lib.mul_f32, C.c_float

        al, bt = cv(alpha), cv(beta)
        bp, cp = b.data, out.data

        def run(stream):
            fn(h, bp, ldb, cp, ldc, ncol, al, bt, stream)

        k = Kernel(run, mats=[a, b, out], name='mul',
                   meta=dict(a=a, b=b, out=out, alpha=alpha, beta=beta,
                             nnz=nnz, op=host))
        return k
