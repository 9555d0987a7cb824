"""Matrices, views, kernels and graphs of the ``b200`` backend.

The semantics mirror the reference backend API
(``pyfr/backends/base/types.py:19-533``): matrices are allocated inside
named extents (one device allocation per extent, zero-filled), carry an
io-shape and an AoSoA device layout with a SoA block of 32 elements
(``pyfr/backends/cuda/base.py:55-59``), views describe gathers of
interface points through an element-offset map, and graphs hold a set of
kernels with dependencies that are topologically ordered on commit.

Execution differs from the reference in one way that matters for speed:
a committed graph is captured once as a CUDA graph by stream capture and
replayed with a single launch; binding a new runtime scalar (``t``,
``dt``) marks the capture stale and it is re-recorded on the next run.
"""

from bisect import insort
from collections import defaultdict
import ctypes as C

import numpy as np

SOASZ = 32


# --------------------------------------------------------------------------
# Layout helpers (pure numpy; testable without a GPU)
# --------------------------------------------------------------------------

def layout(ioshape, tags, soasz=SOASZ, csubsz=SOASZ):
    """(nrow, ncol, leaddim, datashape) of a matrix with ``ioshape``.

    2-D matrices are plain row-major with the leading dimension padded to
    ``csubsz`` when tagged 'align'; 3-D (nrow, nvar, narr) and 4-D
    (n0, n1, nvar, narr) matrices are AoSoA with narr padded to ``csubsz``
    (``pyfr/backends/base/types.py:52-75`` with blocks=False).
    """
    shape, ndim = list(ioshape), len(ioshape)
    if ndim == 2:
        nrow, ncol = shape
        ldmod = csubsz if 'align' in tags else 1
        leaddim = ncol - (ncol % -ldmod)
        datashape = [1, nrow, leaddim]
    elif ndim in (3, 4):
        nvar, narr = shape[-2], shape[-1]
        nparr = narr - narr % -csubsz
        nrow = shape[0] if ndim == 3 else shape[0]*shape[1]
        ncol = nvar*nparr
        leaddim = ncol
        datashape = [1, *shape[:-2], nparr // soasz, nvar, soasz]
    else:
        raise ValueError(f'Unsupported matrix rank {ndim}')

    return nrow, ncol, leaddim, datashape


def pack(ary, nrow, leaddim, soasz=SOASZ, csubsz=SOASZ):
    """io-shape array -> device layout (flat, nrow*leaddim)."""
    n = ary.shape[-1]
    if ary.ndim == 2:
        ary = np.pad(ary, [(0, 0), (0, -n % leaddim if leaddim else 0)])
        ary = ary[:, :leaddim]
    else:
        ary = np.pad(ary, [(0, 0)]*(ary.ndim - 1) + [(0, -n % csubsz)])
        ary = ary.reshape(ary.shape[:-1] + (-1, soasz)).swapaxes(-2, -3)

    return np.ascontiguousarray(ary).reshape(nrow, leaddim)


def unpack(flat, ioshape, datashape):
    """Device layout -> io-shape array."""
    ary = flat.reshape(datashape)
    if len(ioshape) == 2:
        return ary[0, :, :ioshape[1]]

    ary = ary[0].swapaxes(-2, -3)
    ary = ary.reshape(tuple(ioshape[:-1]) + (-1,))
    return ary[..., :ioshape[-1]]


def view_mapping(mats, matmap, rmap, cmap, nvcol, soasz=SOASZ):
    """Element offsets (from the shared storage base) of each view point:
    matrix offset + row*leaddim + AoSoA column displacement
    (``pyfr/backends/base/types.py:285-310``, blocks=False)."""
    n = len(matmap)
    offset = np.empty(n, dtype=np.int64)
    leaddim = np.empty(n, dtype=np.int64)
    for mid, m in mats.items():
        ix = np.where(matmap == mid)
        offset[ix] = m.offset // m.itemsize
        leaddim[ix] = m.leaddim

    rowdisp = np.asarray(rmap, dtype=np.int64)*leaddim
    cmap = np.asarray(cmap, dtype=np.int64)
    coldisp = (cmap // soasz)*soasz*nvcol + cmap % soasz
    return offset + rowdisp + coldisp, leaddim


# --------------------------------------------------------------------------
# Storage
# --------------------------------------------------------------------------

class Extent:
    """A named group of matrices sharing one device allocation."""

    def __init__(self, name=None):
        self.name = name
        self.nbytes = 0
        self.basedata = None
        self._pending = []
        self.storage_root = self

    def reserve(self, obj, nbytes):
        self._pending.append((obj, self.nbytes))
        self.nbytes += nbytes

    def commit(self, alloc_fn):
        self.basedata = alloc_fn(self.nbytes)
        for obj, off in self._pending:
            obj.onalloc(self.basedata, off)
            obj.storage_root = self
        self._pending.clear()


class MatrixBase:
    _base_tags = frozenset()

    def __init__(self, backend, dtype, ioshape, initval, extent, tags):
        self.backend = backend
        self.tags = set(self._base_tags) | set(tags)
        self.dtype = np.dtype(dtype)
        self.itemsize = self.dtype.itemsize
        self.ioshape = tuple(int(s) for s in ioshape)

        (self.nrow, self.ncol, self.leaddim,
         self.datashape) = layout(self.ioshape, self.tags, backend.soasz,
                                  backend.csubsz)
        self.nblocks = 1
        self.blocksz = self.nrow*self.leaddim
        self.nbytes = self.blocksz*self.itemsize
        self.traits = (1, self.nrow, self.ncol, self.leaddim, self.dtype)

        if initval is not None:
            initval = np.asanyarray(initval)
            if initval.shape != self.ioshape:
                raise ValueError('Invalid initial value')
            self._initval = np.asarray(initval, dtype=self.dtype)
        else:
            self._initval = None

        self.basedata = None
        self.offset = 0
        backend.malloc(self, extent)

    def onalloc(self, basedata, offset):
        self.basedata = basedata
        self.offset = offset
        self.data = basedata + offset

        if self._initval is not None:
            self._set(self._initval)
        del self._initval

    @property
    def _as_parameter_(self):
        return self.data

    @property
    def allocated(self):
        return self.basedata is not None

    def get(self):
        if not self.allocated:
            if self._initval is not None:
                return self._initval
            return np.zeros(self.ioshape, dtype=self.dtype)

        flat = np.empty((self.nrow, self.leaddim), dtype=self.dtype)
        self.backend.memcpy_dtoh(flat, self.data, self.nbytes)
        return unpack(flat, self.ioshape, self.datashape).copy()

    def _set(self, ary):
        buf = pack(np.asarray(ary, dtype=self.dtype), self.nrow, self.leaddim,
                   self.backend.soasz, self.backend.csubsz)
        self.backend.memcpy_htod(self.data, buf, self.nbytes)

    def slice(self, ra=None, rb=None, ca=None, cb=None):
        ra, rb = ra or 0, self.nrow if rb is None else rb
        ca, cb = ca or 0, self.ncol if cb is None else cb
        return self.backend.matrix_slice(self, ra, rb, ca, cb)


class Matrix(MatrixBase):
    def set(self, ary):
        ary = np.asanyarray(ary)
        if ary.shape != self.ioshape:
            raise ValueError('Invalid matrix shape')

        if not self.allocated:
            self._initval = np.asarray(ary, dtype=self.dtype)
        else:
            self._set(ary)


class ConstMatrix(MatrixBase):
    _base_tags = frozenset({'const'})

    def __init__(self, backend, dtype, initval, tags):
        super().__init__(backend, dtype, initval.shape, initval, None, tags)


class XchgMatrix(Matrix):
    _base_tags = frozenset({'xchg'})


class MatrixSlice:
    def __init__(self, backend, mat, ra, rb, ca, cb):
        if ra < 0 or rb > mat.nrow or rb < ra:
            raise ValueError('Invalid row slice')
        if ca < 0 or cb > mat.ncol or cb < ca:
            raise ValueError('Invalid column slice')
        if ca % backend.soasz:
            raise ValueError('Starting column must conform to backend '
                             'alignment requirements')

        self.backend = backend
        self.parent = mat
        self.ra, self.rb, self.ca, self.cb = int(ra), int(rb), int(ca), int(cb)
        self.nrow, self.ncol = self.rb - self.ra, self.cb - self.ca
        self.dtype, self.itemsize = mat.dtype, mat.itemsize
        self.leaddim, self.blocksz = mat.leaddim, mat.blocksz
        self.nblocks = 1
        self.traits = (1, self.nrow, self.ncol, self.leaddim, self.dtype)
        self.tags = set(mat.tags) | {'slice'}
        self.ioshape = getattr(mat, 'ioshape', None)

        if ca == 0 and cb == mat.ncol:
            self.nbytes = self.nrow*self.leaddim*self.itemsize

    @property
    def basedata(self):
        return self.parent.basedata

    @property
    def offset(self):
        return self.parent.offset + (self.ra*self.leaddim + self.ca)*self.itemsize

    @property
    def data(self):
        return self.basedata + self.offset

    @property
    def _as_parameter_(self):
        return self.data

    @property
    def storage_root(self):
        return self.parent.storage_root


class View:
    """Gather of interface points: (matrix, row, column) triples turned
    into element offsets from the common storage base."""

    def __init__(self, backend, matmap, rmap, cmap, rstridemap, vshape, tags):
        matmap = np.asarray(matmap)
        self.n = len(matmap)
        self.nvrow = vshape[-2] if len(vshape) == 2 else 1
        self.nvcol = vshape[-1] if len(vshape) >= 1 else 1

        mats = {int(i): backend.mats[int(i)] for i in np.unique(matmap)}
        first = next(iter(mats.values())) if mats else None
        if first is None:
            raise ValueError('Empty view')

        if any(m.storage_root is not first.storage_root
               for m in mats.values()):
            raise TypeError('All viewed matrices must belong to the same '
                            'storage object')
        if any(m.dtype != first.dtype for m in mats.values()):
            raise TypeError('Mixed data types are not supported')

        self.basedata = first.basedata
        self.refdtype = first.dtype

        mapping, leaddim = view_mapping(mats, matmap, rmap, cmap, self.nvcol,
                                        backend.soasz)
        ixdtype = backend.ixdtype
        if ixdtype == np.int32 and mapping.size and mapping.max() >= 2**31:
            raise RuntimeError('View offsets overflow the normal memory model')

        self.mapping = backend.const_matrix(mapping.astype(ixdtype)[None, :],
                                            dtype=ixdtype, tags=tags)
        if self.nvrow > 1:
            rstrides = (np.asarray(rstridemap)*leaddim).astype(ixdtype)[None, :]
            self.rstrides_val = int(rstrides.flat[0])
            self.rstrides = backend.const_matrix(rstrides, dtype=ixdtype,
                                                 tags=tags)
        else:
            self.rstrides_val = 0
            self.rstrides = None


class XchgView:
    def __init__(self, backend, matmap, rmap, cmap, rstridemap, vshape, tags):
        self.view = backend.view(matmap, rmap, cmap, rstridemap, vshape, tags)
        self.n = self.view.n
        self.nvrow, self.nvcol = self.view.nvrow, self.view.nvcol
        self.xchgmat = backend.xchg_matrix((self.nvrow, self.nvcol*self.n),
                                           tags=tags)


# --------------------------------------------------------------------------
# Kernels
# --------------------------------------------------------------------------

class Kernel:
    """A launchable unit; ``run(stream)`` enqueues it."""
    compound = False
    rtnames = ()

    def __init__(self, fn=None, mats=(), views=(), misc=(), name=None,
                 meta=None):
        self._fn = fn
        self.mats = list(mats)
        self.views = list(views)
        self.misc = list(misc)
        self.dt = float('nan')
        self.name = name
        self.meta = meta or {}
        self.graphs = set()

    @property
    def retval(self):
        return None

    def run(self, stream):
        if self._fn is not None:
            self._fn(stream)

    def _mark_stale(self):
        for g in list(self.graphs):
            g.stale = True


class BindableKernel(Kernel):
    """Kernel with runtime-bindable scalar arguments (``rtnames``)."""

    def __init__(self, fn, rtnames, defaults=None, **kwargs):
        super().__init__(fn, **kwargs)
        self.rtnames = tuple(rtnames)
        self.rtargs = dict(defaults or {})

    def bind(self, *args, **kwargs):
        kwargs |= dict(zip(self.rtnames, args))
        changed = False
        for k, v in kwargs.items():
            if k in self.rtnames and self.rtargs.get(k) != v:
                self.rtargs[k] = v
                changed = True
        if changed:
            self._mark_stale()

    def run(self, stream):
        self._fn(stream, **self.rtargs)


class NullKernel(Kernel):
    pass


class MetaKernel(Kernel):
    def __init__(self, kernels):
        super().__init__()
        self.kernels = list(kernels)
        bk = [k for k in self.kernels if hasattr(k, 'bind')]
        if bk:
            self._bkerns = bk
            self.rtnames = tuple({n for k in bk for n in k.rtnames})
            self.bind = self._bind

    def _bind(self, *args, **kwargs):
        for k in self._bkerns:
            k.bind(*args, **kwargs)

    def run(self, stream):
        for k in self.kernels:
            k.run(stream)

    @property
    def graphs(self):
        return set()

    @graphs.setter
    def graphs(self, v):
        pass

    def register_graph(self, g):
        for k in self.kernels:
            if hasattr(k, 'register_graph'):
                k.register_graph(g)
            else:
                k.graphs.add(g)


class OrderedMetaKernel(MetaKernel):
    pass


class UnorderedMetaKernel(MetaKernel):
    def __init__(self, kernels, splits=None):
        super().__init__(kernels)
        if splits is not None:
            self.splits = list(splits)
            self.compound = True
            if len(self.splits) != len(self.kernels) - 1:
                raise ValueError('Invalid split points')


# --------------------------------------------------------------------------
# Graphs
# --------------------------------------------------------------------------

class Graph:
    """A DAG of kernels (``pyfr/backends/base/types.py:343-533``).

    ``group(kerns, subs)`` records fusion hints: the backend's fuser may
    replace a recognised group with a single fused kernel on commit.
    """

    def __init__(self, backend):
        self.backend = backend
        self.committed = False
        self._pkerns = []
        self.kdeps = {}
        self.kpdeps = {}
        self._pgroups = []
        self.klist = []
        self.stale = True
        self._gexec = None
        self.use_cuda_graph = backend.use_cuda_graphs

    def add(self, kern, deps=[], pdeps=[]):
        if self.committed:
            raise RuntimeError('Can not add nodes to a committed graph')
        if kern in self.kdeps:
            raise RuntimeError('Can only add a kernel to a graph once')

        self._pkerns.append(kern)
        self.kdeps[kern] = list(deps)
        self.kpdeps[kern] = list(pdeps)

    def add_all(self, kerns, deps=[], pdeps=[]):
        for k in kerns:
            self.add(k, deps, pdeps)

    def add_mpi_req(self, req, deps=[]):
        raise RuntimeError('MPI requests are not supported by the b200 '
                           'backend (single GPU)')

    def add_mpi_reqs(self, reqs, deps=[]):
        for r in reqs:
            self.add_mpi_req(r, deps)

    def group(self, kerns, subs=[]):
        if self.committed:
            raise RuntimeError('Can not group kernels in a committed graph')
        self._pgroups.append((list(kerns), list(subs)))

    def _topo_sort(self):
        # Kahn's algorithm keyed on insertion order; groups stay contiguous
        grouped = {}
        for kerns, _ in self._pgroups:
            for k in kerns:
                grouped.setdefault(k, kerns[0])
        sup = lambda k: grouped.get(k, k)
        members = defaultdict(list)
        for k in self._pkerns:
            members[sup(k)].append(k)

        order = {k: i for i, k in enumerate(self._pkerns)}
        snodes = list(members)
        key = lambda s: min(order[m] for m in members[s])

        succ, indeg = defaultdict(set), {s: 0 for s in snodes}
        for s in snodes:
            ds = {sup(d) for m in members[s]
                  for d in self.kdeps[m] + self.kpdeps[m]
                  if d in self.kdeps} - {s}
            indeg[s] = len(ds)
            for d in ds:
                succ[d].add(s)

        ready = sorted((s for s in snodes if not indeg[s]), key=key)
        out = []
        while ready:
            s = ready.pop(0)
            out.extend(sorted(members[s], key=order.get))
            for t in succ[s]:
                indeg[t] -= 1
                if not indeg[t]:
                    insort(ready, t, key=key)

        if len(out) != len(self._pkerns):
            raise RuntimeError('Cycle in kernel graph')
        return out

    def commit(self):
        self.committed = True
        klist = self._topo_sort()
        self.klist = self.backend.fuse(klist, self._pgroups)
        for k in self.klist:
            if hasattr(k, 'register_graph'):
                k.register_graph(self)
            else:
                k.graphs.add(self)
        self.stale = True

    def run(self, stream):
        if not self.use_cuda_graph:
            for k in self.klist:
                k.run(stream)
            return

        if self.stale or self._gexec is None:
            self.backend.release_gexec(self._gexec)
            self._gexec = self.backend.capture(
                lambda s: [k.run(s) for k in self.klist], stream)
            self.stale = False

        self.backend.lib.graph_launch(self._gexec, stream)

    def __del__(self):
        try:
            self.backend.release_gexec(self._gexec)
        except Exception:
            pass
