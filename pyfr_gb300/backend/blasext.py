"""BLAS-like extension kernels (``pyfr/backends/base/blasext.py:8-46``):
``axnpby``, ``copy``, ``zero`` and the ``errest`` reduction used for the
PI controller's error norm.
"""

import ctypes as C

import numpy as np

from pyfr_gb300.backend.types import BindableKernel, Kernel


class ErrestKernel(BindableKernel):
    """Device reduction whose scalar result is read back by ``retval``."""

    def __init__(self, fn, out, host, **kwargs):
        super().__init__(fn, ['rtol'], {'rtol': 0.0}, **kwargs)
        self._out = out
        self._host = host

    @property
    def retval(self):
        return [float(self._host[0])]


class ReductionKernel(Kernel):
    """Device reduction to one value, read back by ``retval``."""

    def __init__(self, fn, host, **kwargs):
        super().__init__(fn, **kwargs)
        self._host = host

    @property
    def retval(self):
        return [float(self._host[0])]


class BlasExtKernels:
    MAX_ERREST_BLOCKS = 4096

    def __init__(self, backend):
        self.backend = backend
        self._scratch = None

    @property
    def _sfx(self):
        return 'f64' if self.backend.fpdtype == np.float64 else 'f32'

    def axnpby(self, *arr, in_scale=(), in_scale_idxs=(), out_scale=()):
        if any(arr[0].traits != x.traits for x in arr[1:]):
            raise ValueError('Incompatible matrix types')
        if in_scale or out_scale:
            raise NotImplementedError('Scaled axnpby is not provided')

        be, nv = self.backend, len(arr)
        n = arr[0].nrow*arr[0].leaddim
        fn = getattr(be.lib, f'axnpby_{self._sfx}')
        ptrs = (C.c_void_p*nv)(*[a.data for a in arr])
        coeffs = (C.c_double*nv)()

        def run(stream, **kw):
            for i in range(nv):
                coeffs[i] = kw[f'a{i}']
            fn(n, nv, arr[0].data, ptrs, coeffs, stream)

        return BindableKernel(run, [f'a{i}' for i in range(nv)],
                              {f'a{i}': 0.0 for i in range(nv)},
                              mats=list(arr), misc=[ptrs, coeffs],
                              name='axnpby')

    def copy(self, dst, src):
        if dst.traits != src.traits:
            raise ValueError('Incompatible matrix types')
        be, nbytes = self.backend, dst.nrow*dst.leaddim*dst.itemsize
        dp, sp = dst.data, src.data

        def run(stream):
            be.lib.memcpy_dtod(dp, sp, nbytes, stream)

        return Kernel(run, mats=[dst, src], name='copy')

    def zero(self, m):
        be, nbytes = self.backend, m.nrow*m.leaddim*m.itemsize
        p = m.data

        def run(stream):
            be.lib.memset(p, 0, nbytes, stream)

        return Kernel(run, mats=[m], name='zero')

    def reduction(self, rop, exprs, vvars, svars=None, pvars=None):
        """``reduction(rop, exprs, vvars)`` of
        pyfr/backends/base/blasext.py:21-46 for the form the CFL controller
        uses (pyfr/solvers/baseadvec/system.py:48-52): the maximum of one
        variable, ``exprs == [name]`` with ``vvars == {name: matrix}``.
        Other operators and expressions are not provided."""
        if rop != 'max' or len(exprs) != 1 or exprs[0] not in vvars or \
                len(vvars) != 1 or svars or pvars:
            raise NotImplementedError('Only the maximum of one variable is '
                                      'provided')
        be, x = self.backend, vvars[exprs[0]]
        n = x.nrow*x.leaddim if x.nrow > 1 else x.ncol
        fn = be.lib.reduce_max_f64 if x.dtype == np.float64 else \
            be.lib.reduce_max_f32
        out = be.matrix((1, 2), dtype=np.float64)
        be.commit()
        host = np.zeros(1)
        xp, kp = x.data, out.data
        op = out.data + 8

        def run(stream):
            fn(n, xp, kp, op, stream)
            be.lib.memcpy_dtoh(host.ctypes.data, op, 8, stream)

        return ReductionKernel(run, host, mats=[x, out], name='reduction')

    def errest(self, curr, err, atols, norm='l2', uref=None, hcoef=0.0):
        """Error norm of the PI controller over one element type's
        registers of io-shape (nupts, nvars, neles).  With ``uref`` (one
        FP64 value per variable) the current solution is stored as q with
        u_v = uref_v + q_v (plus hcoef*q_0 for the last variable), and the
        norm scales with |u|."""
        be = self.backend
        nupts, nvars, neles = curr.ioshape
        if curr.traits != err.traits:
            raise ValueError('Incompatible matrix types')

        if self._scratch is None:
            self._scratch = be.matrix((1, self.MAX_ERREST_BLOCKS),
                                      dtype=np.float64)
            be.commit()
        atol = be.const_matrix(np.asarray(atols, dtype=np.float64)[None, :],
                               dtype=np.float64)
        out = be.matrix((1, 1), dtype=np.float64)
        be.commit()

        host = np.zeros(1)
        uniform = int(norm == 'uniform')
        ld, sp, nsc = curr.leaddim, self._scratch.data, self.MAX_ERREST_BLOCKS
        cp, ep, ap, op = curr.data, err.data, atol.data, out.data

        if uref is not None:
            if curr.dtype != np.float64:
                raise ValueError('A shifted error norm needs FP64 registers')
            uref = np.ascontiguousarray(uref, dtype=np.float64)
            if uref.shape != (nvars,):
                raise ValueError('uref needs one value per variable')
            shifted, pu = be.lib.errest_shifted_f64, uref.ctypes.data

            def fn(*a):
                shifted(*a[:9], pu, hcoef, *a[9:])
        elif curr.dtype == np.float64:
            fn = be.lib.errest_f64
        else:
            fn = be.lib.errest_f32

        def run(stream, rtol):
            fn(nupts, nvars, neles, ld, cp, ep, ap, rtol, uniform, sp, nsc, op,
               stream)
            be.lib.memcpy_dtoh(host.ctypes.data, op, 8, stream)

        k = ErrestKernel(run, out, host, mats=[curr, err, atol, out],
                         name='errest')
        k._uref = uref
        return k
