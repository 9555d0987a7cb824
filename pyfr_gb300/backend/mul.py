"""The ``mul`` kernel providers: out = alpha*A@B + beta*out.

Same contract as the reference's GiMMiK/cuBLASLt providers
(``pyfr/backends/cuda/gimmik.py:23-38``): A must be a constant matrix, a
shape mismatch raises ValueError, and a provider that cannot serve a call
raises NotSuitableError so that the backend tries the next one
(``pyfr/backends/base/backend.py:188-216``).

* ``TensorMulKernels``: split-BF16 (three products) tcgen05 kernel for
  single-precision data, selected by ``[backend-b200] mul-precision =
  bf16x3``; declines operators whose tiles do not fit in shared memory.
* ``MulKernels``: sparse (CSR) kernel in the backend's precision, FP64 or
  FP32; always suitable.

Operator data is uploaded once per (matrix, provider) and shared by every
kernel that applies it.
"""

import ctypes as C
import weakref

import numpy as np

from pyfr_gb300.backend.lib import B200Error
from pyfr_gb300.backend.types import Kernel


def _check_shapes(a, b, out):
    if a.ncol != b.nrow or a.nrow != out.nrow or b.ncol != out.ncol:
        raise ValueError('Incompatible matrices for out = a*b')
    if 'const' not in a.tags:
        raise ValueError('The operator of mul must be a constant matrix')


def _destroy_handles(destroy, handles):
    for h in handles.values():
        if h is not None:
            destroy(h[0])
    handles.clear()


class MulKernels:
    def __init__(self, backend):
        from pyfr_gb300.backend.base import release
        self.backend = backend
        self._handles = {}
        weakref.finalize(self, release, _destroy_handles,
                         backend.lib.mul_destroy, self._handles)

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
        _check_shapes(a, b, out)

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

        return Kernel(run, mats=[a, b, out], name='mul',
                      meta=dict(a=a, b=b, out=out, alpha=alpha, beta=beta,
                                nnz=nnz, op=host, impl='csr'))


class TensorMulKernels:
    def __init__(self, backend):
        from pyfr_gb300.backend.base import release
        self.backend = backend
        self._handles = {}
        weakref.finalize(self, release, _destroy_handles,
                         backend.lib.mul_bf16x3_destroy, self._handles)

    def _handle(self, a):
        from pyfr_gb300.backend.base import NotSuitableError

        key = a.mid
        if key not in self._handles:
            host = np.ascontiguousarray(a._host, dtype=np.float64)
            h, smem = C.c_void_p(), C.c_size_t()
            try:
                self.backend.lib.mul_bf16x3_create(
                    host.ctypes.data_as(C.POINTER(C.c_double)), host.shape[0],
                    host.shape[1], C.byref(h), C.byref(smem))
            except B200Error:
                self._handles[key] = None
            else:
                self._handles[key] = (h.value, smem.value, host)

        if self._handles[key] is None:
            raise NotSuitableError('operator too large for the tensor tiles')
        return self._handles[key]

    def mul(self, a, b, out, alpha=1.0, beta=0.0):
        from pyfr_gb300.backend.base import NotSuitableError

        be = self.backend
        if be.fpdtype != np.float32 or be.mul_precision != 'bf16x3':
            raise NotSuitableError('tensor-core mul serves bf16x3 FP32 data')
        _check_shapes(a, b, out)
        if b.leaddim % 4 or out.leaddim % 4 or b.ncol % 4:
            raise NotSuitableError('unaligned operands')
        if beta not in (0.0, 1.0):
            raise NotSuitableError('the tensor-core epilogue stores or adds')

        h, smem, host = self._handle(a)
        ncol, ldb, ldc = b.ncol, b.leaddim, out.leaddim
        al, bt = C.c_float(alpha), C.c_float(beta)
        bp, cp = b.data, out.data
        err = be.status_word
        fn = be.lib.mul_bf16x3

        def run(stream):
            fn(h, bp, ldb, cp, ldc, ncol, al, bt, err, stream)

        return Kernel(run, mats=[a, b, out], name='mul',
                      meta=dict(a=a, b=b, out=out, alpha=alpha, beta=beta,
                                op=host, impl='bf16x3', smem=smem))
