"""Native mesh (``.pyfrm``) and solution (``.pyfrs``) files.

The records follow the reference's format revision 2
(``doc/src/file_format.rst``; writer ``pyfr/readers/base.py:62-105`` and
``pyfr/writers/native.py:178-235,376-410``; reader
``pyfr/readers/native.py:89-520``):

* mesh: ``codec`` (null-padded strings ``eles/<type>``,
  ``eles/<type>/face/<n>``, ``bc/<name>``, ``tag/<name>``), ``creator``,
  ``mesh-uuid``, ``version`` = 2, ``nodes`` (compound ``location``,
  ``valency``), ``eles/<type>`` (compound ``nodes``, ``curved``,
  ``faces[(cidx, off)]``, ``colour``, ``tags``; attribute ``pts``),
  ``periodic/<name>`` (pairs of (cidx, off)) and
  ``partitionings/<n>/eles`` (attribute ``regions``);
* solution: ``config``, ``config-<n>``, ``stats`` (INI text; ``[data]
  prefix``), ``mesh-uuid``, ``creator``, ``version``, serialised state
  (``intg/...``), and per element type ``<prefix>/p<order>-<type>``: one
  compound record per element with the groups ``soln`` (one (nupts,) field
  per conserved variable) and ``aux`` (``part-id``); attribute ``pts``.

The reference stores these records in HDF5 through h5py.  Neither h5py nor
libhdf5 is part of this toolchain, so files written here hold the same
records, under the same paths, in a NumPy ``.npz`` archive (one ``.npy``
member per dataset, ``<path>@<attr>`` per attribute; the structured dtypes
are stored as they are).  A file that starts with the HDF5 signature is
read through h5py when it is importable, so the reference's own files load
where h5py exists; otherwise reading one raises.
"""

from dataclasses import dataclass, field
import hashlib
import os
from pathlib import Path
import re
import uuid as _uuid

import numpy as np

from pyfr_gb300.inifile import Inifile
from pyfr_gb300.mesh import Mesh, Side, face_vertices

FORMAT_VERSION = 2
CREATOR = 'pyfr_gb300 0.1'

# Element types in the order the reference's importer lays them out in the
# codec (ascending Gmsh element-type numbers, pyfr/readers/base.py:363-383)
CODEC_ETYPE_ORDER = ['tri', 'quad', 'tet', 'hex', 'pri', 'pyr']

FACE_DTYPE = np.dtype([('cidx', np.int16), ('off', np.int64)])

_HDF5_SIGNATURE = b'\x89HDF\r\n\x1a\n'


# ---- container ---------------------------------------------------------------

class NativeFile:
    """Read access to the records of a native file by HDF5-style path:
    ``f[path]`` (an array), ``f.attrs(path)`` (a dict), ``path in f`` (a
    dataset or group) and ``f.names(group)`` (a group's members)."""

    def __init__(self, path):
        self.path = str(path)
        with open(path, 'rb') as fh:
            sig = fh.read(8)

        if sig == _HDF5_SIGNATURE:
            try:
                import h5py
            except ImportError:
                raise RuntimeError(f'{path} is an HDF5 file; reading it '
                                   'needs h5py, which is not installed') \
                    from None
            self._h5 = h5py.File(path, 'r')
            self._npz = None
        else:
            self._h5 = None
            self._npz = np.load(path, allow_pickle=False)
            self._dsets = [k for k in self._npz.files if '@' not in k]

    def close(self):
        (self._h5 or self._npz).close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __getitem__(self, name):
        if self._h5 is not None:
            return self._h5[name][()]
        return self._npz[name]

    def __contains__(self, name):
        if self._h5 is not None:
            return name in self._h5
        return name in self._dsets or \
            any(k.startswith(name + '/') for k in self._dsets)

    def attrs(self, name):
        if self._h5 is not None:
            return dict(self._h5[name].attrs)
        pre = name + '@'
        return {k[len(pre):]: self._npz[k] for k in self._npz.files
                if k.startswith(pre)}

    def names(self, group=''):
        """Immediate members of ``group`` (datasets and sub-groups)."""
        if self._h5 is not None:
            return list(self._h5[group or '/'])
        pre = group + '/' if group else ''
        out = []
        for k in self._dsets:
            if k.startswith(pre):
                n = k[len(pre):].split('/')[0]
                if n not in out:
                    out.append(n)
        return out

    def string(self, name):
        v = self[name]
        v = v.item() if isinstance(v, np.ndarray) else v
        return v.decode() if isinstance(v, bytes) else str(v)


class NativeFileWriter:
    """Builds the records of a native file and writes them in one piece
    (to a temporary name that is then moved into place, as the reference's
    writer does, ``pyfr/writers/native.py:247-262``)."""

    def __init__(self):
        self._recs = {}

    def __setitem__(self, name, value):
        if isinstance(value, str):
            value = np.array(value.encode(), dtype='S')
        self._recs[name] = np.asarray(value)

    def __getitem__(self, name):
        return self._recs[name]

    def set_attr(self, name, key, value):
        if name not in self._recs:
            raise KeyError(f'No dataset {name!r}')
        self._recs[f'{name}@{key}'] = np.asarray(value)

    def save(self, path):
        path = Path(path)
        tmp = path.with_name(f'.{path.name}.{_uuid.uuid4().hex}.tmp')
        with open(tmp, 'wb') as fh:
            np.savez(fh, **self._recs)
        os.replace(tmp, path)


# ---- standard elements -------------------------------------------------------

def std_ele(etype, order):
    """Equi-spaced nodes of the standard element of ``etype`` at ``order``
    in the format's node order: x counts quickest, then y, then z
    (``doc/src/file_format.rst`` node ordering; ``pyfr/shapes.py``
    ``std_ele``)."""
    t = np.linspace(-1, 1, order + 1)
    if etype == 'quad':
        return np.array([(x, y) for y in t for x in t])
    if etype == 'hex':
        return np.array([(x, y, z) for z in t for y in t for x in t])
    if etype == 'tri':
        return np.array([(t[i], t[j]) for j in range(order + 1)
                         for i in range(order + 1 - j)])
    if etype == 'tet':
        return np.array([(t[i], t[j], t[k]) for k in range(order + 1)
                         for j in range(order + 1 - k)
                         for i in range(order + 1 - j - k)])
    if etype == 'pri':
        return np.array([(t[i], t[j], z) for z in t
                         for j in range(order + 1)
                         for i in range(order + 1 - j)])
    if etype == 'pyr':
        # Layer k at z = -1 + 2k/order holds (order + 1 - k)^2 nodes at
        # x, y = -1 + (k + 2m)/order (pyfr/shapes.py:618-626)
        return np.array([(-1 + (k + 2*i)/order, -1 + (k + 2*j)/order,
                          -1 + 2*k/order)
                         for k in range(order + 1)
                         for j in range(order + 1 - k)
                         for i in range(order + 1 - k)], dtype=float)
    raise ValueError(f'Unknown element type {etype!r}')


def _order_from_nnodes(etype, n):
    for k in range(1, 32):
        m = len(std_ele(etype, k))
        if m == n:
            return k
        if m > n:
            break
    raise ValueError(f'{n} is not a node count of {etype}')


def corner_nodes(etype, order):
    """Indices of the first-order vertices among the nodes of order
    ``order``, in vertex order."""
    from pyfr_gb300.shapes import VERTICES
    pts = std_ele(etype, order)
    return [int(np.flatnonzero(np.all(np.abs(pts - v) < 1e-12, axis=1))[0])
            for v in np.array(VERTICES[etype], dtype=float)]


# ---- mesh --------------------------------------------------------------------

def _codec(etypes, bcnames, tags=('fluid',)):
    codec = []
    for et in sorted(etypes, key=CODEC_ETYPE_ORDER.index):
        codec.append(f'eles/{et}')
        codec.extend(f'eles/{et}/face/{i}'
                     for i in range(len(face_vertices(et))))
    codec.extend(f'bc/{b}' for b in bcnames)
    codec.extend(f'tag/{t}' for t in tags)
    return codec


def ele_dtype(nnodes, nfaces):
    return np.dtype([('nodes', np.int64, (nnodes,)), ('curved', bool),
                     ('faces', FACE_DTYPE, (nfaces,)), ('colour', np.uint8),
                     ('tags', np.uint64)])


def colour_elements(eles, codec):
    """Greedy colouring of the element graph across interior faces: each
    element, in codec order, takes the least-used colour not held by an
    already coloured neighbour, preferring the smallest available colour
    when the counts tie (``pyfr/readers/base.py:310-361``).  Fills
    ``colour`` in place."""
    order = [et for et in (c[5:] for c in codec if c.count('/') == 1
                           and c.startswith('eles/')) if et in eles]
    disp, d = {}, 0
    for et in order:
        disp[et] = d
        d += len(eles[et])
    cdisp = {}
    for et in order:
        for i in range(eles[et]['faces'].shape[1]):
            cdisp[codec.index(f'eles/{et}/face/{i}')] = disp[et]

    ncol = max(eles[et]['faces'].shape[1] for et in order) + 1
    colours = np.zeros(d, dtype=np.int64)
    counts = [0]*ncol
    for et in order:
        fc = eles[et]['faces']
        cidx, off = fc['cidx'].astype(np.int64), fc['off']
        for e in range(len(fc)):
            g = disp[et] + e
            avail = [True]*ncol
            for c, o in zip(cidx[e], off[e]):
                if o >= 0 and c in cdisp and cdisp[c] + o < g:
                    avail[colours[cdisp[c] + o]] = False
            col = avail.index(True)
            best = counts[col]
            for c in range(ncol):
                if avail[c] and counts[c] and counts[c] < best:
                    col, best = c, counts[c]
            colours[g] = col
            counts[col] += 1
        eles[et]['colour'] = colours[disp[et]:disp[et] + len(fc)]


def mesh_uuid(nodes, eles, codec, pmap):
    """Identifier of a mesh: the first 128 bits of the SHA-256 of its
    records (node table, element arrays in codec order, codec, periodic
    pairs), as a UUID string.  (The reference hashes a pickle of the same
    records, ``pyfr/readers/base.py:66-69``; only equality of a mesh's and
    its solutions' identifiers is ever used.)"""
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(nodes).tobytes())
    for et in sorted(eles, key=CODEC_ETYPE_ORDER.index):
        h.update(et.encode())
        h.update(np.ascontiguousarray(eles[et]).tobytes())
    h.update('\0'.join(codec).encode())
    for k in sorted(pmap):
        h.update(k.encode())
        h.update(np.ascontiguousarray(pmap[k]).tobytes())
    return str(_uuid.UUID(h.hexdigest()[:32]))


def write_mesh(fname, nodes, eles, codec, pmap=None):
    """Write a mesh from its raw records: ``nodes`` (nnodes, ndims),
    ``eles`` {etype: ele_dtype array with nodes, curved, faces filled},
    ``codec`` and periodic pairs ``pmap`` {name: (n, 2) FACE_DTYPE}.
    Computes valencies, the colouring, the default partitioning (curved
    elements first, ``pyfr/readers/base.py:20-47``) and the identifier;
    returns the identifier."""
    pmap = pmap or {}
    nodes = np.asarray(nodes, dtype=np.float64)
    colour_elements(eles, codec)
    uuid = mesh_uuid(nodes, eles, codec, pmap)

    ndims = nodes.shape[1]
    ntab = np.zeros(len(nodes), dtype=[('location', np.float64, (ndims,)),
                                       ('valency', np.uint16)])
    ntab['location'] = nodes
    for einfo in eles.values():
        k, v = np.unique(einfo['nodes'], return_counts=True)
        ntab['valency'][k] += v.astype(np.uint16)

    w = NativeFileWriter()
    w['codec'] = np.array([c.encode() for c in codec], dtype='S')
    w['creator'] = CREATOR
    w['mesh-uuid'] = uuid
    w['version'] = np.int64(FORMAT_VERSION)
    w['nodes'] = ntab
    for et, einfo in eles.items():
        w[f'eles/{et}'] = einfo
        order = _order_from_nnodes(et, einfo['nodes'].shape[1])
        w.set_attr(f'eles/{et}', 'pts', std_ele(et, order))
    for name, pairs in pmap.items():
        w[f'periodic/{name}'] = pairs

    parts, regions = [], [0]
    for et in sorted(eles):
        cur = eles[et]['curved']
        parts.extend([np.flatnonzero(cur), np.flatnonzero(~cur)])
        regions.append(regions[-1] + len(cur))
    w['partitionings/1/eles'] = np.concatenate(parts).astype(np.int64)
    w.set_attr('partitionings/1/eles', 'regions',
               np.array([regions], dtype=np.int64))
    w.save(fname)
    return uuid


def mesh_records(mesh, tol=1e-9):
    """Raw records (nodes, eles, codec, pmap) of a generated linear mesh:
    coincident vertices become one node; interfaces whose two faces do not
    share their nodes are periodic and are grouped by their translation
    into ``periodic/<n>``."""
    from pyfr_gb300.shapes import VERTICES

    etypes = [et for et in CODEC_ETYPE_ORDER if et in mesh.spts]
    allpts = np.concatenate([mesh.spts[et].reshape(-1, mesh.ndims)
                             for et in etypes])
    scale = max(np.ptp(allpts, axis=0).max(), 1.0)
    q = np.rint(allpts / (tol*scale)).astype(np.int64)
    _, first, inv = np.unique(q, axis=0, return_index=True,
                              return_inverse=True)
    nodes = allpts[np.sort(first)]
    # Renumber nodes by first appearance
    remap = np.empty(len(first), dtype=np.int64)
    remap[np.argsort(first)] = np.arange(len(first))
    nid = remap[inv.ravel()]

    codec = _codec(etypes, list(mesh.bcon))
    eles, off = {}, 0
    for et in etypes:
        sp = mesh.spts[et]
        nv, ne = sp.shape[:2]
        if nv != len(VERTICES[et]):
            raise ValueError('Only linear meshes can be converted')
        nf = len(face_vertices(et))
        a = np.zeros(ne, dtype=ele_dtype(nv, nf))
        a['nodes'] = nid[off:off + nv*ne].reshape(nv, ne).T
        a['curved'] = mesh.spts_curved.get(et, np.zeros(ne, bool))
        a['faces']['cidx'] = -1
        a['faces']['off'] = -1
        a['tags'] = 1
        eles[et] = a
        off += nv*ne

    def fcidx(et, f):
        return codec.index(f'eles/{et}/face/{f}')

    lhs, rhs = mesh.con
    let, lei, lfi = lhs.etypes.tolist(), lhs.eidxs, lhs.fidxs
    ret, rei, rfi = rhs.etypes.tolist(), rhs.eidxs, rhs.fidxs
    for i in range(len(lhs)):
        eles[let[i]]['faces'][lei[i], lfi[i]] = (fcidx(ret[i], rfi[i]), rei[i])
        eles[ret[i]]['faces'][rei[i], rfi[i]] = (fcidx(let[i], lfi[i]), lei[i])
    for name, sd in mesh.bcon.items():
        c = codec.index(f'bc/{name}')
        for et, e, f in zip(sd.etypes.tolist(), sd.eidxs, sd.fidxs):
            eles[et]['faces'][e, f] = (c, -1)
    for et, a in eles.items():
        if np.any(a['faces']['cidx'] < 0):
            raise ValueError('Mesh has faces with no neighbour or boundary')

    # Periodic interfaces: faces with different node sets
    def fnodes(et, e, f):
        return eles[et]['nodes'][e, face_vertices(et)[f]]

    def fcen(et, e, f):
        return mesh.spts[et][face_vertices(et)[f], e].mean(axis=0)

    groups = {}
    for i in range(len(lhs)):
        ln = np.sort(fnodes(let[i], lei[i], lfi[i]))
        rn = np.sort(fnodes(ret[i], rei[i], rfi[i]))
        if np.array_equal(ln, rn):
            continue
        t = fcen(ret[i], rei[i], rfi[i]) - fcen(let[i], lei[i], lfi[i])
        tq = np.rint(t / (tol*scale)).astype(np.int64)
        lf = (fcidx(let[i], lfi[i]), lei[i])
        rf = (fcidx(ret[i], rfi[i]), rei[i])
        # Orient each group so that its translation's first nonzero
        # component is positive (left faces on the low side)
        nz = tq[np.flatnonzero(tq)[0]]
        if nz < 0:
            tq, lf, rf = -tq, rf, lf
        groups.setdefault(tuple(tq.tolist()), []).append((lf, rf))
    pmap = {str(k): np.array([[(int(a), int(b)) for a, b in pr]
                              for pr in groups[t]], dtype=FACE_DTYPE)
            for k, t in enumerate(sorted(groups))}
    return nodes, eles, codec, pmap


def save_mesh(fname, mesh):
    """Write a generated mesh as a native mesh file; returns its
    identifier."""
    return write_mesh(fname, *mesh_records(mesh))


def _select_partitioning(f, pname):
    if pname is not None:
        path = f'partitionings/{pname}/eles'
        regions = f.attrs(path)['regions']
        if len(regions) != 1:
            raise RuntimeError(f'Partitioning {pname} has {len(regions)} '
                               'parts but running with 1 rank')
        return path, regions
    for name in f.names('partitionings'):
        path = f'partitionings/{name}/eles'
        regions = f.attrs(path)['regions']
        if len(regions) == 1:
            return path, regions
    raise RuntimeError('Mesh does not have any partitionings with 1 rank')


def read_mesh(fname, pname=None):
    """Read a native mesh file into a ``Mesh`` (one partition).

    Elements of each type are numbered in the partition's order
    (``mesh.eidxs[etype]`` holds their numbers in the file); interior
    interfaces are the paired faces of the ``faces`` arrays with each pair
    kept once, its left side the face met first in (type, face, element)
    order, and boundaries come from the ``bc/<name>`` codec entries
    (``pyfr/readers/native.py:281-466``)."""
    from pyfr_gb300.shapes import VERTICES

    with NativeFile(fname) as f:
        version = int(f['version'])
        if version != FORMAT_VERSION:
            raise RuntimeError(f'Mesh file must be format v{FORMAT_VERSION}')
        codec = [c.decode() for c in f['codec']]
        uuid = f.string('mesh-uuid')
        creator = f.string('creator')
        etypes = sorted(f.names('eles'))

        ppath, regions = _select_partitioning(f, pname)
        peles = f[ppath]
        reg = regions[0]
        eidxs = {et: peles[reg[i]:reg[i + 1]] for i, et in enumerate(etypes)
                 if reg[i + 1] > reg[i]}

        nodes = f['nodes']
        ndims = nodes.dtype['location'].shape[0]
        eles = {et: f[f'eles/{et}'][eidxs[et]] for et in eidxs}

    spts, curved, colours, tags, snodes = {}, {}, {}, {}, {}
    for et, einfo in eles.items():
        if np.any(einfo['curved']):
            raise NotImplementedError('Curved elements are not supported: '
                                      'the geometry path is linear')
        nn = einfo['nodes'].shape[1]
        cn = corner_nodes(et, _order_from_nnodes(et, nn)) \
            if nn != len(VERTICES[et]) else slice(None)
        locs = nodes['location'][einfo['nodes'][:, cn]]   # (neles, nv, nd)
        spts[et] = np.ascontiguousarray(locs.swapaxes(0, 1))
        curved[et] = np.zeros(len(einfo), dtype=bool)
        colours[et] = einfo['colour']
        tags[et] = einfo['tags']
        snodes[et] = einfo['nodes']

    # Codec entries of element faces
    cidxmap = {}
    for cidx, c in enumerate(codec):
        if (m := re.match(r'eles/(\w+)/face/(\d+)$', c)):
            cidxmap[cidx] = (m[1], int(m[2]))

    # Global-to-local element numbers
    g2l = {}
    for et, gi in eidxs.items():
        m = np.full(int(gi.max()) + 1 if len(gi) else 0, -1, dtype=np.int64)
        m[gi] = np.arange(len(gi))
        g2l[et] = m

    lc, le, rc, re_ = [], [], [], []
    for et, einfo in eles.items():
        for fidx, eface in enumerate(einfo['faces'].T):
            lc.append(np.full(len(eface), codec.index(f'eles/{et}/face/{fidx}'),
                              dtype=np.int64))
            le.append(np.arange(len(eface)))
            rc.append(eface['cidx'].astype(np.int64))
            re_.append(eface['off'].astype(np.int64))
    lc, le, rc, rg = map(np.concatenate, (lc, le, rc, re_))

    # Local numbers of the right-hand elements (-1 for boundaries)
    rl = np.full(len(rc), -1, dtype=np.int64)
    for cidx, (et, _) in cidxmap.items():
        mask = (rc == cidx) & (rg >= 0)
        if np.any(mask):
            m = g2l[et]
            ok = rg[mask] < len(m)
            vals = np.full(mask.sum(), -1, dtype=np.int64)
            vals[ok] = m[rg[mask][ok]]
            rl[mask] = vals
    isbc = rg == -1
    islocal = rl >= 0
    if np.any(~(isbc | islocal)):
        raise RuntimeError('Mesh faces refer to elements outside the '
                           'partition')

    stride = max(int(le.max(initial=-1)), int(rl.max(initial=-1))) + 1
    lkey = lc[islocal]*stride + le[islocal]
    rkey = rc[islocal]*stride + rl[islocal]
    keep = np.flatnonzero(islocal)[lkey < rkey]

    def side(c, e):
        et = np.array([cidxmap[int(x)][0] for x in c])
        fi = np.array([cidxmap[int(x)][1] for x in c], dtype=np.int64)
        return Side(et, e, fi)

    con = (side(lc[keep], le[keep]), side(rc[keep], rl[keep]))
    bcon = {}
    for bc in np.unique(rc[isbc]):
        name = codec[bc]
        if not name.startswith('bc/'):
            raise RuntimeError(f'Boundary face with codec entry {name!r}')
        m = rc == bc
        bcon[name[3:]] = side(lc[m], le[m])

    return Mesh(ndims=ndims, spts=spts, con=con, spts_curved=curved,
                bcon=bcon, uuid=uuid, codec=codec, eidxs=eidxs,
                fname=str(fname), creator=creator, colours=colours,
                tags=tags, spts_nodes=snodes)


# ---- solutions ---------------------------------------------------------------

@dataclass
class Solution:
    """A solution file's records (``pyfr/readers/native.py:50-58``): the
    configuration and statistics INI files, the field names, per element
    type the data (nupts, nvars, neles) in the mesh's local element order
    and the auxiliary fields, the earlier configurations and the
    serialised state."""
    config: object
    stats: object
    fields: list
    data: dict = field(default_factory=dict)
    aux: dict = field(default_factory=dict)
    prevcfgs: dict = field(default_factory=dict)
    state: dict = field(default_factory=dict)
    uuid: str = None
    grad_data: dict = field(default_factory=dict)


def soln_dtype(fields, nupts, fpdtype, aux=(), ndims=0):
    """Nested compound dtype of one element's solution record
    (``pyfr/writers/native.py:222-235``); with ``ndims`` a ``grad`` group
    of (ndims, nupts) per field."""
    groups = [('soln', [(n, fpdtype, (nupts,)) for n in fields])]
    if ndims:
        groups.append(('grad', [(n, fpdtype, (ndims, nupts))
                                for n in fields]))
    afields = [('part-id', np.int64)] + list(aux)
    return np.dtype(groups + [('aux', afields)])


def write_soln(fname, mesh, data, upts, fields, config, stats, *,
               prefix='soln', prevcfgs=None, state=None, fpdtype=None,
               grads=None, subset=None):
    """Write a solution file.

    ``data`` maps element types to (nupts, nvars, neles) arrays in the
    mesh's local element order; they are stored at the elements' numbers
    in the mesh file (``mesh.eidxs``, else in local order).  ``upts`` maps
    element types to their solution points; ``config`` is the current
    Inifile and ``prevcfgs`` the {'config-<n>': INI text} history, to which
    the current configuration is appended when it differs from the last
    entry (``pyfr/integrators/base.py:369-381``); ``state`` holds
    serialised arrays such as ``intg/ctrl``; ``grads`` maps element types
    to their physical gradients (ndims, nupts, nvars, neles); ``subset``
    maps element types to the local elements to write (the others are
    left out and a ``<key>-idxs`` array lists the elements' numbers,
    ascending, ``pyfr/writers/native.py:237-245``)."""
    order = config.getint('solver', 'order')
    w = NativeFileWriter()
    cfgtxt = config.tostr()
    chain = dict(prevcfgs or {})
    n = len(chain)
    if n == 0 or chain.get(f'config-{n - 1}') != cfgtxt:
        chain[f'config-{n}'] = cfgtxt
    w['config'] = cfgtxt
    for k, v in chain.items():
        w[k] = v
    stats = stats or Inifile()
    if not stats.hasopt('data', 'prefix'):
        stats.set('data', 'prefix', prefix)
    w['stats'] = stats.tostr()
    w['mesh-uuid'] = mesh.uuid or ''
    w['creator'] = CREATOR
    w['version'] = np.int64(FORMAT_VERSION)
    for k, v in (state or {}).items():
        w[k] = np.asarray(v)

    for et, u in data.items():
        u = np.asarray(u)
        nupts, nvars, neles = u.shape
        g = None if grads is None else np.asarray(grads[et])
        dt = soln_dtype(fields, nupts, fpdtype or u.dtype,
                        ndims=0 if g is None else g.shape[0])
        gi = (mesh.eidxs or {}).get(et)
        gi = np.arange(neles) if gi is None else np.asarray(gi)
        sel = np.arange(neles) if subset is None or et not in subset else \
            np.asarray(subset[et], dtype=np.int64)
        # Records in ascending order of the elements' numbers
        o = np.argsort(gi[sel], kind='stable')
        sel, nums = sel[o], gi[sel][o]
        if subset is None and len(nums) and int(nums[-1]) + 1 != len(nums):
            raise ValueError('Element numbers do not cover the mesh')
        arr = np.zeros(len(sel), dtype=dt)
        for i, name in enumerate(fields):
            arr['soln'][name] = u[:, i, sel].T
            if g is not None:
                arr['grad'][name] = g[:, :, i, sel].transpose(2, 0, 1)
        ek = f'{prefix}/p{order}-{et}'
        w[ek] = arr
        w.set_attr(ek, 'pts', np.asarray(upts[et], dtype=np.float64))
        if subset is not None and et in subset:
            w[f'{ek}-idxs'] = nums.astype(np.int64)
    w.save(fname)


def read_soln(fname, mesh, prefix=None):
    """Read a solution file written for ``mesh`` (identifiers must agree;
    ``pyfr/readers/native.py:113-235``).  Subset solutions raise (a
    restart needs every element); ``read_subset_soln`` reads them."""
    return _read_soln(fname, mesh, prefix, False)[1]


def read_subset_soln(fname, mesh, prefix=None):
    """(mesh, solution) of a solution file that may hold a subset of the
    elements: the mesh is then cut down to the elements present, in their
    order in the file, and has no interfaces
    (``pyfr/readers/native.py:196-271``)."""
    return _read_soln(fname, mesh, prefix, True)


def _read_soln(fname, mesh, prefix, allow_subset):
    with NativeFile(fname) as f:
        uuid = f.string('mesh-uuid')
        if mesh.uuid is not None and uuid != mesh.uuid:
            raise RuntimeError('Invalid solution for mesh')
        if int(f['version']) != FORMAT_VERSION:
            raise RuntimeError(f'Solution file must be format '
                               f'v{FORMAT_VERSION}')
        top = f.names()
        cfgs = {k: Inifile(f.string(k)) for k in top
                if k.startswith('config')}
        stats = Inifile(f.string('stats'))
        state = {}
        for g in ('plugins', 'bcs', 'intg'):
            if g in top:
                for n in f.names(g):
                    state[f'{g}/{n}'] = f[f'{g}/{n}']

        soln = Solution(config=cfgs['config'], stats=stats, fields=None,
                        prevcfgs={k: v for k, v in cfgs.items()
                                  if k.startswith('config-')},
                        state=state, uuid=uuid)
        order = soln.config.getint('solver', 'order')
        prefix = prefix or stats.get('data', 'prefix')
        subset = {}
        for et in mesh.etypes:
            ek = f'{prefix}/p{order}-{et}'
            gi = (mesh.eidxs or {}).get(et)
            gi = np.arange(mesh.spts[et].shape[1]) if gi is None else gi
            if ek not in f or f'{ek}-idxs' in f:
                if not allow_subset:
                    raise RuntimeError('Subset solutions are not supported'
                                       if ek in f else
                                       f'Solution has no {ek}')
                if ek not in f:
                    subset[et] = np.empty(0, dtype=np.int64)
                    continue
                nums = f[f'{ek}-idxs']
                # Local elements of the file's element numbers
                pos = np.full(int(max(gi.max(), nums.max())) + 1, -1)
                pos[gi] = np.arange(len(gi))
                if (pos[nums] < 0).any():
                    raise ValueError(f'{ek}-idxs names elements that are '
                                     'not in the mesh')
                subset[et] = pos[nums]
                rec = f[ek]
            else:
                rec = f[ek][gi]
            names = list(rec.dtype['soln'].names)
            if soln.fields is None:
                soln.fields = names
            u = np.stack([rec['soln'][n] for n in names], axis=1)
            soln.data[et] = np.ascontiguousarray(u.transpose(2, 1, 0))
            soln.aux[et] = {n: rec['aux'][n] for n in rec.dtype['aux'].names}
            if 'grad' in rec.dtype.names:
                g = np.stack([rec['grad'][n] for n in names], axis=1)
                # (neles, nvars, ndims, nupts) -> (ndims, nupts, nvars, neles)
                soln.grad_data[et] = np.ascontiguousarray(
                    g.transpose(2, 3, 1, 0))

    if not subset:
        return mesh, soln
    from dataclasses import replace
    spts, eidxs, curved = {}, {}, {}
    for et in mesh.etypes:
        sel = subset.get(et)
        gi = (mesh.eidxs or {}).get(et)
        gi = np.arange(mesh.spts[et].shape[1]) if gi is None else gi
        cv = (mesh.spts_curved or {}).get(et)
        cv = np.zeros(mesh.spts[et].shape[1], bool) if cv is None else cv
        if sel is None:
            spts[et], eidxs[et], curved[et] = mesh.spts[et], gi, cv
        elif len(sel):
            spts[et], eidxs[et] = mesh.spts[et][:, sel], gi[sel]
            # (curved flags follow their elements, as the reference's
            # _subset_mesh keeps them: pyfr/readers/native.py:255-271)
            curved[et] = cv[sel]
    sub = replace(mesh, spts=spts, eidxs=eidxs, con=None, bcon={},
                  spts_curved=curved)
    soln.data = {et: v for et, v in soln.data.items() if et in spts}
    return sub, soln


def file_path_gen(basedir, basename):
    """Output paths: ``basename`` formatted with the time ``t`` and the
    output count ``n`` (``pyfr/util.py:180-201``)."""
    n = 0
    t = yield
    while True:
        t = yield Path(basedir) / basename.format(t=t, n=n)
        n += 1
