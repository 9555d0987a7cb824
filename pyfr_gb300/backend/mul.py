"""The ``mul`` kernel providers: out = alpha*A@B + beta*out.

Same contract as the reference's GiMMiK/cuBLASLt providers
(``pyfr/backends/cuda/gimmik.py:23-38``): A must be a constant matrix, a
shape mismatch raises ValueError, and a provider that cannot serve a call
raises NotSuitableError so that the backend tries the next one
(``pyfr/backends/base/backend.py:188-216``).

* ``TensorMulKernels``: split-BF16 (three products) tcgen05 kernel for
  single-precision data, selected by ``[backend-b200] mul-precision =
  bf16x3``; declines operators whose tiles do not fit in shared memory.
  It also provides the fused ``mul_cat`` and ``mul_batched`` forms.
* ``MulKernels``: sparse (CSR) kernel in the backend's precision, FP64 or
  FP32; always suitable.

Operator data is uploaded once per (matrix, provider) and shared by every
kernel that applies it.
"""

import ctypes as C
import json
import os
import weakref

import numpy as np

from pyfr_gb300.backend.lib import B200Error, MulArgs
from pyfr_gb300.backend.types import Kernel


def _check_shapes(a, b, out):
    if a.ncol != b.nrow or a.nrow != out.nrow or b.ncol != out.ncol:
        raise ValueError('Incompatible matrices for out = a*b')
    if 'const' not in a.tags:
        raise ValueError('The operator of mul must be a constant matrix')


_PLANS = None


def _plan_path():
    root = os.environ.get('PYFR_GB300_CACHE',
                          os.path.join(os.path.expanduser('~'), '.cache',
                                       'pyfr_gb300'))
    return os.path.join(root, 'mul-plans.json')


def _plan_cache():
    global _PLANS
    if _PLANS is None:
        try:
            with open(_plan_path()) as f:
                _PLANS = json.load(f)
        except (OSError, ValueError):
            _PLANS = {}
    return _PLANS


def _save_plan_cache():
    try:
        path = _plan_path()
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = f'{path}.{os.getpid()}'
        with open(tmp, 'w') as f:
            json.dump(_PLANS, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def _destroy_handles(destroy, handles):
    # (entries are handle tuples, failures (None) and piece lists)
    for h in handles.values():
        if isinstance(h, tuple):
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
    """Split-BF16 tcgen05 operator applies (``mul``) plus the fused forms
    the Navier-Stokes graph uses in the chosen precision form:

    * ``mul_cat(a1, b1, a2, b2, out, alpha, beta, rowscale)``:
      out = alpha*S*(a1@b1 + a2@b2) + beta*out with S the optional
      per-(row, element) scale ``rowscale`` (an (m, neles) matrix);
    * ``mul_batched(a, b, out, nbatch)``: out_z = a@b_z over nbatch equal
      row slices of b and out.

    Operator data is uploaded once per operator (or operator pair)."""

    def __init__(self, backend):
        from pyfr_gb300.backend.base import release
        self.backend = backend
        self._handles = {}
        self._nterms = {}
        weakref.finalize(self, release, _destroy_handles,
                         backend.lib.mul_bf16x3_destroy, self._handles)

    def _suitable(self):
        from pyfr_gb300.backend.base import NotSuitableError

        be = self.backend
        if be.fpdtype != np.float32 or be.mul_precision not in ('bf16x3',
                                                                'tf32'):
            raise NotSuitableError('tensor-core mul serves bf16x3 or tf32 '
                                   'FP32 data')

    MAX_ROWS = 256          # UMMA N limit of one handle (operator rows)

    def _handle_arrays(self, key, hosts):
        """Handle of the K-concatenation of one or two FP64 operator blocks
        (host arrays of equal row count), cached under ``key``; None when no
        pipeline plan fits shared memory."""
        if key not in self._handles:
            a1 = np.ascontiguousarray(hosts[0], dtype=np.float64)
            a2 = np.ascontiguousarray(hosts[1], dtype=np.float64) \
                if len(hosts) > 1 else None
            h, smem = C.c_void_p(), C.c_size_t()
            pd = C.POINTER(C.c_double)
            lib = self.backend.lib
            tf32 = self.backend.mul_precision == 'tf32'
            args = (a1.ctypes.data_as(pd), a1.shape[1],
                    a2.ctypes.data_as(pd) if a2 is not None else None,
                    a2.shape[1] if a2 is not None else 0, a1.shape[0])

            # Five products need the operator in three terms; where that
            # image leaves no room for the ring, two terms and four products
            want = 3 if self.backend.split_products == 5 and not tf32 else 2
            self._handles[key] = None
            if a1.shape[0] <= self.MAX_ROWS:
                for nterms in range(want, 1, -1):
                    try:
                        plan = self._tuned_plan(args, tf32, nterms) \
                            if self.backend.autotune else None
                        lib.mul_tc_create_terms(*args, int(tf32), nterms,
                                                *(plan or (0, 0)),
                                                C.byref(h), C.byref(smem))
                    except B200Error:
                        continue
                    self._handles[key] = (h.value, smem.value,
                                          [a1] + ([a2] if a2 is not None
                                                  else []))
                    self._nterms[h.value] = nterms
                    break
        return self._handles[key]

    def _pieces(self, ops):
        """Cover the operator [A1 | A2] (constant matrices of equal row
        count) with handles that fit: a list of (r0, r1, blocks, handle),
        blocks being up to two (operator index, k0, k1) column ranges.
        The whole operator when it fits, else row ranges of at most
        MAX_ROWS rows, each split along K into 32-aligned ranges until
        every piece fits."""
        from pyfr_gb300.backend.base import NotSuitableError

        key = tuple(a.mid for a in ops)
        if ('pieces', key) in self._handles:
            return self._handles['pieces', key]

        hosts = [np.ascontiguousarray(a._host, dtype=np.float64) for a in ops]
        m = hosts[0].shape[0]
        whole = [(i, 0, h.shape[1]) for i, h in enumerate(hosts)]
        h = self._handle_arrays(key, hosts)
        if h is not None:
            pieces = [(0, m, whole, h)]
        else:
            pieces = []
            nr = -(-m // self.MAX_ROWS)
            step = -(-(-(-m // nr)) // 32)*32
            for r0 in range(0, m, step):
                r1 = min(m, r0 + step)
                queue = list(whole)
                while queue:
                    cand = queue[:2]
                    while True:
                        subs = [hosts[i][r0:r1, k0:k1] for i, k0, k1 in cand]
                        hk = key + ((r0, r1),) + tuple(cand)
                        h = self._handle_arrays(hk, subs)
                        if h is not None:
                            break
                        if len(cand) == 2:
                            cand = cand[:1]
                            continue
                        i, k0, k1 = cand[0]
                        if k1 - k0 <= 32:
                            self._handles['pieces', key] = None
                            raise NotSuitableError('operator too large for '
                                                   'the tensor tiles')
                        mid = k0 + -(-((k1 - k0)//2) // 32)*32
                        queue[0:1] = [(i, k0, mid), (i, mid, k1)]
                        cand = queue[:1]
                    pieces.append((r0, r1, cand, h))
                    del queue[:len(cand)]
        self._handles['pieces', key] = pieces
        return pieces

    def _build(self, ops, bs, out, alpha, beta, rowscale=None, nbatch=1,
               bstrides=(0, 0), cstride=0, meta=None):
        """The kernel applying [A1 | A2] to [B1; B2] piece by piece: each row
        range's first piece stores (or adds, with beta = 1), the others
        add; the row scale applies to every piece (it is linear)."""
        from pyfr_gb300.backend.base import NotSuitableError

        pieces = self._pieces(ops)
        if pieces is None:
            raise NotSuitableError('operator too large for the tensor tiles')
        isz = 4
        nvars = ldr = 0
        if rowscale is not None:
            nvars, ldr = out.ioshape[1], rowscale.leaddim
            # One scale per element when every row holds the same (1/|J|
            # of affine elements): the epilogue loads it once per column
            uni = self._uniform_rows(rowscale)
            if uni is not None:
                rowscale, ldr = uni, 0
        arglist, seen = [], set()
        for r0, r1, blocks, (h, smem, hosts) in pieces:
            first = r0 not in seen
            seen.add(r0)
            bp = [bs[i].data + k0*bs[i].leaddim*isz for i, k0, _ in blocks]
            a = MulArgs(b1=bp[0], ldb1=bs[blocks[0][0]].leaddim,
                        b2=bp[1] if len(bp) > 1 else None,
                        ldb2=bs[blocks[1][0]].leaddim if len(bp) > 1 else 0,
                        c=out.data + r0*out.leaddim*isz, ldc=out.leaddim,
                        ncol=out.ncol, nbatch=nbatch,
                        bstride1=bstrides[blocks[0][0]],
                        bstride2=bstrides[blocks[1][0]] if len(bp) > 1 else 0,
                        cstride=cstride, alpha=alpha,
                        beta=beta if first else 1.0,
                        rowscale=(rowscale.data + r0*ldr*isz
                                  if rowscale is not None else None),
                        ldr=ldr, nvars=nvars)
            arglist.append((h, a))

        meta = dict(meta or {}, smem=max(p[3][1] for p in pieces),
                    pieces=len(pieces))
        if len(pieces) == 1:
            h, a = arglist[0]
            return self._kernel(h, a, list(ops) + list(bs) + [out] +
                                ([rowscale] if rowscale is not None else []),
                                meta)

        be = self.backend
        for h, a in arglist:
            a.err = be.status_word
            a.products = self._products(self._nterms.get(h, 2))
        meta['products'] = min(a.products for _, a in arglist)
        if be.mul_precision == 'tf32':
            meta['impl'] = meta['impl'].replace('bf16x3', 'tf32')
        fn = be.lib.mul_bf16x3_apply
        calls = [(h, C.addressof(a)) for h, a in arglist]

        def run(stream):
            for h, pa in calls:
                fn(h, pa, stream)

        k = Kernel(run, mats=list(ops) + list(bs) + [out] +
                   ([rowscale] if rowscale is not None else []),
                   misc=[a for _, a in arglist], name='mul', meta=meta)
        return k

    def _handle(self, *ops):
        from pyfr_gb300.backend.base import NotSuitableError

        key = tuple(a.mid for a in ops)
        h = self._handle_arrays(key, [a._host for a in ops])
        if h is None:
            raise NotSuitableError('operator too large for the tensor tiles')
        return h

    @staticmethod
    def _aligned(*mats):
        return all(m.leaddim % 4 == 0 for m in mats)

    def _products(self, nterms):
        p = self.backend.split_products
        return 5 if nterms == 3 else min(p, 4)

    def _tuned_plan(self, args, tf32, nterms=2):
        """Pipeline plan (ring stages, epilogue staging tiles) of an
        operator, picked by timing every plan that fits on a
        representative width (8 tiles of 128 columns per SM) and cached per
        device and operator, in memory and in a JSON file
        (``$PYFR_GB300_CACHE`` or ``~/.cache/pyfr_gb300``)."""
        be, lib = self.backend, self.backend.lib
        m, k1, k2 = args[4], args[1], args[3]
        # (plans of kernels with rings of any length)
        key = '|'.join(map(str, (be.platform_id, 'tf32' if tf32 else 'bf16',
                                 self._products(nterms), m, k1, k2, 'r2')))
        cache = _plan_cache()
        if key in cache:
            return tuple(cache[key]) if cache[key] else None

        sms = C.c_int()
        lib.device_info(C.byref(sms), None, None, None, None, None, 0)
        ncol = sms.value*128*8
        bufs = []

        def dev(nbytes):
            p = C.c_void_p()
            lib.malloc(C.byref(p), nbytes)
            bufs.append(p.value)
            return p.value

        b1, c = dev(4*k1*ncol), dev(4*m*ncol)
        b2 = dev(4*k2*ncol) if k2 else None
        err = be.status_word
        ev0, ev1 = C.c_void_p(), C.c_void_p()
        lib.event_create(C.byref(ev0))
        lib.event_create(C.byref(ev1))
        times = {}
        try:
            for ntiles in (1, 2):
                for nstages in range(4, 11):
                    h, smem = C.c_void_p(), C.c_size_t()
                    try:
                        lib.mul_tc_create_terms(*args, int(tf32), nterms,
                                                nstages, ntiles, C.byref(h),
                                                C.byref(smem))
                    except B200Error:
                        continue
                    a = MulArgs(b1=b1, ldb1=ncol, b2=b2, ldb2=ncol, c=c,
                                ldc=ncol, ncol=ncol, nbatch=1, alpha=1.0,
                                beta=0.0, products=self._products(nterms),
                                err=err)
                    pa = C.addressof(a)
                    for _ in range(2):
                        lib.mul_bf16x3_apply(h.value, pa, be.stream)
                    lib.event_record(ev0.value, be.stream)
                    for _ in range(5):
                        lib.mul_bf16x3_apply(h.value, pa, be.stream)
                    lib.event_record(ev1.value, be.stream)
                    lib.event_sync(ev1.value)
                    ms = C.c_float()
                    lib.event_elapsed(C.byref(ms), ev0.value, ev1.value)
                    times[(nstages, ntiles)] = ms.value
                    lib.mul_bf16x3_destroy(h.value)
        finally:
            for p in bufs:
                lib.free(p)
            lib.event_destroy(ev0.value)
            lib.event_destroy(ev1.value)
        be.check_status()

        best = min(times, key=times.get) if times else None
        cache[key] = list(best) if best else None
        _save_plan_cache()
        return best

    def _kernel(self, handle, args, mats, meta):
        be = self.backend
        args.err = be.status_word
        args.products = self._products(self._nterms.get(handle, 2))
        meta['products'] = args.products
        if be.mul_precision == 'tf32':
            meta['impl'] = meta['impl'].replace('bf16x3', 'tf32')
        fn = be.lib.mul_bf16x3_apply
        pa = C.addressof(args)

        def run(stream):
            fn(handle, pa, stream)

        k = Kernel(run, mats=mats, name='mul', meta=meta)
        k._args = args
        k._handle = handle
        return k

    def with_stage(self, k, acc, u, a, b, last, dt=0.0, dtdev=None):
        """A copy of the one-piece apply ``k`` whose epilogue performs the
        mixed-precision two-register RK stage instead of storing its output
        R: acc += dt*b*R (FP64) and the next FP32 input u = fl32(acc_old) +
        fl32(dt*a)*R, or fl32(acc_new) at the last stage (the arithmetic of
        ``b200_rkmixed_f64f32``, bit for bit).  acc and u have the output's
        layout.  None when ``k`` cannot take it (several pieces, slices, an
        accumulating output)."""
        args = getattr(k, '_args', None)
        out = k.meta.get('out')
        if args is None or args.nbatch != 1 or args.beta != 0.0 or \
                out is None or acc.leaddim != out.leaddim or \
                u.leaddim != out.leaddim or acc.nrow != out.nrow:
            return None
        new = MulArgs()
        C.memmove(C.addressof(new), C.addressof(args), C.sizeof(MulArgs))
        new.rk_acc, new.rk_u = acc.data, u.data
        new.rk_dt_dev = dtdev.data if dtdev is not None else None
        new.rk_dt, new.rk_a, new.rk_b = dt, a, b
        new.rk_stage = 2 if last else 1
        fn, h = self.backend.lib.mul_bf16x3_apply, k._handle
        pa = C.addressof(new)

        def run(stream):
            fn(h, pa, stream)

        kk = Kernel(run, mats=list(k.mats) + [acc, u], misc=[new], name='mul',
                    meta=dict(k.meta, rk_stage=new.rk_stage, acc=acc, u=u))
        kk._args = new
        kk._handle = h
        return kk

    def mul(self, a, b, out, alpha=1.0, beta=0.0):
        from pyfr_gb300.backend.base import NotSuitableError

        self._suitable()
        _check_shapes(a, b, out)
        if not self._aligned(b, out) or b.ncol % 4:
            raise NotSuitableError('unaligned operands')
        if beta not in (0.0, 1.0):
            raise NotSuitableError('the tensor-core epilogue stores or adds')

        return self._build([a], [b], out, alpha, beta,
                           meta=dict(a=a, b=b, out=out, alpha=alpha,
                                     beta=beta, op=np.asarray(a._host),
                                     impl='bf16x3'))

    def _uniform_rows(self, rs):
        """The first row of a row-scale matrix as a one-row matrix when
        every row is equal to it (known from the host copy), else None."""
        h = getattr(rs, '_host', None)
        if h is None or h.ndim != 2 or h.shape[0] < 2:
            return None
        key = ('uniform', rs.mid)
        if key not in self._handles:
            # (compared as the kernel reads them: in the matrix's precision)
            hd = np.asarray(h, dtype=rs.dtype)
            same = bool(np.all(hd == hd[:1]))
            self._handles[key] = self.backend.const_matrix(
                hd[:1], dtype=rs.dtype, tags={'align'}) if same else None
        return self._handles[key]

    def mul_cat(self, a1, b1, a2, b2, out, alpha=1.0, beta=0.0,
                rowscale=None):
        from pyfr_gb300.backend.base import NotSuitableError

        self._suitable()
        _check_shapes(a1, b1, out)
        _check_shapes(a2, b2, out)
        if b1.ncol != b2.ncol:
            raise ValueError('Incompatible matrices for out = a1*b1 + a2*b2')
        if not self._aligned(b1, b2, out) or b1.ncol % 4:
            raise NotSuitableError('unaligned operands')
        if beta not in (0.0, 1.0):
            raise NotSuitableError('the tensor-core epilogue stores or adds')
        nvars = ldr = 0
        if rowscale is not None:
            if len(out.ioshape) != 3 or rowscale.nrow != out.nrow:
                raise ValueError('A row scale needs an (nrow, nvars, neles) '
                                 'output and one row per output row')
            nvars, ldr = out.ioshape[1], rowscale.leaddim
            if rowscale.dtype != np.float32:
                raise ValueError('The row scale must be FP32')

        return self._build([a1, a2], [b1, b2], out, alpha, beta,
                           rowscale=rowscale,
                           meta=dict(a=a1, b=b1, a2=a2, b2=b2, out=out,
                                     alpha=alpha, beta=beta,
                                     op=np.asarray(a1._host),
                                     op2=np.asarray(a2._host),
                                     rowscale=rowscale, impl='bf16x3-cat'))

    def mul_batched(self, a, b, out, nbatch, alpha=1.0, beta=0.0):
        from pyfr_gb300.backend.base import NotSuitableError

        self._suitable()
        m, k = a.nrow, a.ncol
        if b.nrow != nbatch*k or out.nrow != nbatch*m or b.ncol != out.ncol:
            raise ValueError('Incompatible matrices for batched out = a*b')
        if 'const' not in a.tags:
            raise ValueError('The operator of mul must be a constant matrix')
        if not self._aligned(b, out) or b.ncol % 4:
            raise NotSuitableError('unaligned operands')
        if beta not in (0.0, 1.0):
            raise NotSuitableError('the tensor-core epilogue stores or adds')

        return self._build([a], [b], out, alpha, beta, nbatch=nbatch,
                           bstrides=(k*b.leaddim, 0), cstride=m*out.leaddim,
                           meta=dict(a=a, b=b, out=out, alpha=alpha,
                                     beta=beta, op=np.asarray(a._host),
                                     nbatch=nbatch, impl='bf16x3-batched'))
