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
        """x0 <- a0 x0 + sum a_i x_i (pyfr/backends/base/blasext.py:9-19),
        with the coefficients bound at run time (a0, a1, ...).  in_scale
        and out_scale are per-variable factors (one per variable of the
        registers' io-shape (..., nvars, neles)): in_scale multiplies the
        terms of the registers listed in in_scale_idxs, out_scale the
        sum."""
        if any(arr[0].traits != x.traits for x in arr[1:]):
            raise ValueError('Incompatible matrix types')

        be, nv = self.backend, len(arr)
        n = arr[0].nrow*arr[0].leaddim
        ptrs = (C.c_void_p*nv)(*[a.data for a in arr])
        coeffs = (C.c_double*nv)()
        if in_scale or out_scale:
            nvars = arr[0].ioshape[-2]
            for sc in (in_scale, out_scale):
                if sc and len(sc) != nvars:
                    raise ValueError('Scales need one value per variable')
            if in_scale and not in_scale_idxs:
                raise ValueError('in_scale needs in_scale_idxs')
            if any(not 0 <= k < nv for k in in_scale_idxs):
                raise ValueError('in_scale_idxs out of range')
            insc = (C.c_double*nvars)(*in_scale) if in_scale else None
            outsc = (C.c_double*nvars)(*out_scale) if out_scale else None
            mask = sum(1 << k for k in in_scale_idxs) if in_scale else 0
            fs = getattr(be.lib, f'axnpby_scaled_{self._sfx}')

            def fn(n, nv, x0, ptrs, coeffs, stream):
                fs(n, nv, nvars, x0, ptrs, coeffs, insc, mask, outsc, stream)
            keep = [insc, outsc]
        else:
            fn, keep = getattr(be.lib, f'axnpby_{self._sfx}'), []

        def run(stream, **kw):
            for i in range(nv):
                coeffs[i] = kw[f'a{i}']
            fn(n, nv, arr[0].data, ptrs, coeffs, stream)

        return BindableKernel(run, [f'a{i}' for i in range(nv)],
                              {f'a{i}': 0.0 for i in range(nv)},
                              mats=list(arr), misc=[ptrs, coeffs, *keep],
                              name='axnpby')

    def copy(self, dst, src):
        if dst.traits != src.traits:
            raise ValueError('Incompatible matrix types')
        be, nbytes = self.backend, dst.nrow*dst.leaddim*dst.itemsize
        dp, sp = dst.data, src.data

        def run(stream):
            be.lib.memcpy_dtod(dp, sp, nbytes, stream)

        return Kernel(run, mats=[dst, src], name='copy')

    def pack_view(self, view, out):
        """Gather the points of ``view`` into the exchange buffer ``out``
        (io-shape (nvrow, nvcol, n)): b200_pack_view_*."""
        if out.ioshape != (view.nvrow, view.nvcol, view.n):
            raise ValueError('Exchange buffer does not match the view')
        be = self.backend
        fn = getattr(be.lib, f'pack_view_{self._sfx}')
        n, nr, nc = view.n, view.nvrow, view.nvcol
        b, m = view.basedata, view.mapping.data
        r = view.rstrides.data if view.rstrides is not None else None
        ix64, op, ld = int(be.ixdtype == np.int64), out.data, out.leaddim

        def run(stream):
            fn(n, nr, nc, b, m, r, ix64, op, ld, stream)

        return Kernel(run, mats=[out], views=[view], name='pack')

    def zero(self, m):
        be, nbytes = self.backend, m.nrow*m.leaddim*m.itemsize
        p = m.data

        def run(stream):
            be.lib.memset(p, 0, nbytes, stream)

        return Kernel(run, mats=[m], name='zero')

    # The error norm of PyFR's PI controller as a reduction expression
    # (pyfr/integrators/controllers.py:105-117): squared and summed for the
    # l2 norm, absolute and maximised for the uniform norm
    _ERR_EXPR = 'err/(atol+rtol*fabs(curr))'

    @classmethod
    def _errest_form(cls, rop, exprs, vvars, svars, pvars):
        """'l2' or 'uniform' when (rop, exprs, ...) is the PI controller's
        error norm over registers curr and err, else None."""
        if len(exprs) != 1 or set(vvars) != {'curr', 'err'} or \
                list(svars or []) != ['rtol'] or set(pvars or {}) != {'atol'}:
            return None
        e, q = exprs[0].replace(' ', ''), cls._ERR_EXPR
        if rop == 'sum' and e == f'({q})*({q})':
            return 'l2'
        if rop == 'max' and e == f'fabs({q})':
            return 'uniform'
        return None

    def reduction(self, rop, exprs, vvars, svars=None, pvars=None):
        """``reduction(rop, exprs, vvars, svars, pvars)`` of
        pyfr/backends/base/blasext.py:21-46 in the forms that PyFR's
        explicit path makes: the PI controller's error norm (l2 or
        uniform; ``retval`` is the sum of squares or the largest value, the
        scalar ``rtol`` bound at run time, ``atol`` one value per variable)
        and the maximum of one variable (the CFL controller's wave speed,
        pyfr/solvers/baseadvec/system.py:48-52).  Other expressions are not
        provided."""
        norm = self._errest_form(rop, exprs, vvars, svars, pvars)
        if norm is not None:
            return self.errest(vvars['curr'], vvars['err'],
                               list(np.ravel(pvars['atol'])), norm=norm)
        if rop != 'max' or len(exprs) != 1 or exprs[0] not in vvars or \
                len(vvars) != 1 or svars or pvars:
            raise NotImplementedError('Reductions other than the error norm '
                                      'and the maximum of one variable are '
                                      'not provided')
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
