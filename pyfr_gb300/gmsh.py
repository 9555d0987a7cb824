"""Gmsh mesh import (ASCII ``.msh`` formats 2.2 and 4.1, first-order
elements) into the native mesh records.

Behaviour of ``pyfr/readers/gmsh.py`` and ``pyfr/readers/base.py:108-497``:

* physical names: a name ``periodic[ _-]<id>[ _-](l|r)`` marks one side of
  the periodic pair ``<id>``; names of the highest dimension are volume
  regions (each becomes a ``tag/<name>`` entry, element tag bits in sorted
  name order); every other name is a boundary (``bc/<name>``).  Names are
  lower-cased; duplicates are errors.
* elements of a volume region make up the mesh, grouped by type in
  ascending Gmsh type number; faces are paired by their vertex sets,
  periodic faces by the fuzzy lexicographic order of their centroids,
  boundary faces by the vertex sets of the boundary's elements; any face
  left over is an error.
* the node table is the dense range of the file's node numbers.

The geometry of this solver is linear: high-order Gmsh elements are read
when they are straight (their nodes on the linear element's lattice) and
kept as their vertices; curved ones raise.
"""

from collections import defaultdict
import re

import numpy as np

from pyfr_gb300.mesh import face_vertices
from pyfr_gb300.native import (CODEC_ETYPE_ORDER, FACE_DTYPE, ele_dtype,
                               write_mesh)

# Gmsh element-type numbers of the first-order elements and their vertex
# counts
GMSH_ETYPES = {1: ('line', 2), 2: ('tri', 3), 3: ('quad', 4), 4: ('tet', 4),
               5: ('hex', 8), 6: ('pri', 6), 7: ('pyr', 5)}

# Gmsh numbers the vertices of a quadrilateral face around the face; the
# native format numbers them x fastest, then y (then z)
GMSH_VERTEX_ORDER = {'line': [0, 1], 'tri': [0, 1, 2], 'quad': [0, 1, 3, 2],
                     'tet': [0, 1, 2, 3], 'hex': [0, 1, 3, 2, 4, 5, 7, 6],
                     'pri': [0, 1, 2, 3, 4, 5], 'pyr': [0, 1, 3, 2, 4]}

# Higher-order Gmsh element types (Gmsh's element-type numbering): native
# type, node count and order.  Gmsh lists the vertices first, in the
# first-order element's order.
GMSH_HIGH_ORDER = {
    8: ('line', 3, 2), 26: ('line', 4, 3), 27: ('line', 5, 4),
    9: ('tri', 6, 2), 21: ('tri', 10, 3), 23: ('tri', 15, 4),
    10: ('quad', 9, 2), 36: ('quad', 16, 3), 37: ('quad', 25, 4),
    11: ('tet', 10, 2), 29: ('tet', 20, 3), 30: ('tet', 35, 4),
    12: ('hex', 27, 2), 92: ('hex', 64, 3), 93: ('hex', 125, 4),
    13: ('pri', 18, 2), 90: ('pri', 40, 3), 91: ('pri', 75, 4)}

# Pyramids of any order and higher-order types without a linear reading
GMSH_UNSUPPORTED = {14, 118, 119}

_NDIMS = {'tri': 2, 'quad': 2, 'tet': 3, 'hex': 3, 'pri': 3, 'pyr': 3}


def fuzzy_lexsort(pts, idx, tol=1e-6):
    """Indices ``idx`` ordered lexicographically by the columns of ``pts``
    (ndims, n), where values of a coordinate that lie within ``tol`` of the
    first value of their run count as equal and the run is ordered by the
    next coordinate (the order of ``pyfr/nputil.py:120-136``)."""
    def rec(ix, d):
        ix = sorted(ix, key=lambda k: pts[d][k])
        if len(ix) < 2 or d + 1 >= len(pts):
            return ix
        out, start = [], 0
        for j in range(1, len(ix) + 1):
            if j == len(ix) or pts[d][ix[j]] - pts[d][ix[start]] >= tol:
                run = ix[start:j]
                out.extend(rec(run, d + 1) if len(run) > 1 else run)
                start = j
        return out

    return rec(list(idx), 0)


class GmshReader:
    def __init__(self, msh):
        if isinstance(msh, str) and '\n' not in msh:
            with open(msh) as fh:
                lines = fh.read().splitlines()
        else:
            text = msh if isinstance(msh, str) else msh.read()
            lines = text.splitlines()

        self._volpents, self._bfacespents = {}, {}
        self._pfacespents = defaultdict(list)
        self._tagpents = {}
        self._version = None

        it = iter(lines)
        readers = {'MeshFormat': self._read_format,
                   'PhysicalNames': self._read_phys_names,
                   'Entities': self._read_entities,
                   'Nodes': self._read_nodes,
                   'Elements': self._read_eles}
        for ln in it:
            if not ln.strip():
                continue
            if not ln.startswith('$'):
                raise ValueError('Expected a mesh section')
            sect = ln[1:].strip()
            if sect in readers:
                readers[sect](it)
                if next(it).strip() != f'$End{sect}':
                    raise ValueError(f'Expected $End{sect}')
            else:
                for el in it:
                    if el.strip() == f'$End{sect}':
                        break
                else:
                    raise ValueError(f'Expected $End{sect}')

        if not self._volpents:
            raise ValueError('No volume elements in mesh')

    # ---- sections ------------------------------------------------------------

    def _read_format(self, it):
        ver, ftype, dsize = next(it).split()
        if ver not in ('2.2', '4.1'):
            raise ValueError('Invalid mesh version')
        if ftype != '0':
            raise ValueError('Invalid file type')
        if dsize != '8':
            raise ValueError('Invalid data size')
        self._version = ver

    def _read_phys_names(self, it):
        n = int(next(it))
        pnames, seen_n, seen_i = [], set(), set()
        for _ in range(n):
            m = re.match(r'(\d+) (\d+) "((?:[^"\\]|\\.)*)"$', next(it).strip())
            if not m:
                raise ValueError('Malformed physical entity')
            dim, pent, name = int(m[1]), int(m[2]), m[3].lower()
            if name in seen_n:
                raise ValueError(f'Duplicate physical name: {name}')
            if pent in seen_i:
                raise ValueError(f'Duplicate physical entity ID: {pent}')
            pnames.append((dim, pent, name))
            seen_n.add(name)
            seen_i.add(pent)

        voldim = max(d for d, _, _ in pnames)
        for dim, pent, name in pnames:
            if name.startswith('periodic'):
                p = re.match(r'periodic[ _-]([a-z0-9]+)[ _-](l|r)$', name)
                if not p:
                    raise ValueError('Invalid periodic boundary condition')
                self._pfacespents[p[1]].append(pent)
            elif dim == voldim:
                self._volpents[name] = pent
            else:
                self._bfacespents[name] = pent

        if any(len(v) != 2 for v in self._pfacespents.values()):
            raise ValueError('Unpaired periodic boundary in mesh')

    def _read_entities(self, it):
        npts, *ents = (int(i) for i in next(it).split())
        for _ in range(npts):
            next(it)
        for ndim, nent in enumerate(ents, start=1):
            for _ in range(nent):
                e = next(it).split()
                etag, nphys = int(e[0]), int(e[7])
                if nphys:
                    self._tagpents[ndim, etag] = tuple(sorted(
                        abs(int(e[8 + i])) for i in range(nphys)))

    def _read_nodes(self, it):
        if self._version == '2.2':
            n = int(next(it))
            rows = [next(it).split() for _ in range(n)]
            ix = np.array([int(r[0]) for r in rows], dtype=np.int64)
            xyz = np.array([[float(v) for v in r[1:4]] for r in rows])
        else:
            ne, nn, lo, hi = (int(i) for i in next(it).split())
            ix, xyz = [], []
            for _ in range(ne):
                cnt = int(next(it).split()[-1])
                ix.extend(int(next(it)) for _ in range(cnt))
                xyz.extend([float(v) for v in next(it).split()[:3]]
                           for _ in range(cnt))
            ix, xyz = np.array(ix, dtype=np.int64), np.array(xyz)
        lo = int(ix.min())
        self._nodepts = np.full((int(ix.max()) - lo + 1, 3), np.nan)
        self._nodepts[ix - lo] = xyz
        self._nodeoff = lo

    def _check_type(self, etype):
        if etype in GMSH_UNSUPPORTED or (etype not in GMSH_ETYPES and
                                         etype not in GMSH_HIGH_ORDER):
            raise ValueError(f'Unsupported element type {etype}')

    def _nnodes(self, etype):
        return GMSH_HIGH_ORDER[etype][1] if etype in GMSH_HIGH_ORDER else \
            GMSH_ETYPES[etype][1]

    LINEARISE_CHUNK = 512

    def _linearise(self, etype, nodes, lintol=1e-5):
        """The vertices of high-order elements whose other nodes all lie on
        the equi-spaced lattice of their linear element (within ``lintol``
        of the element's extent): straight elements stored at a higher
        order (the reference snaps these too, pyfr/readers/base.py:
        464-497).  Curved elements raise: the geometry path is linear."""
        if etype not in GMSH_HIGH_ORDER:
            return etype, nodes
        from pyfr_gb300.native import std_ele
        from pyfr_gb300.shapes import VERTICES, linear_shape_fn
        petype, nn, order = GMSH_HIGH_ORDER[etype]
        lin = {v[0]: k for k, v in GMSH_ETYPES.items()}
        nv = len(VERTICES[petype]) if petype != 'line' else 2
        verts = nodes[:, :nv] - self._nodeoff
        if petype != 'line':
            lat = std_ele(petype, order)
            # Lattice positions from the vertices (Gmsh vertex order ->
            # the format's), in all three coordinates: a boundary face of a
            # 3-D mesh may bend out of its plane in any of them
            sf = linear_shape_fn(petype, lat)                # (nlat, nv)
            vo = GMSH_VERTEX_ORDER[petype]
            # Elements in fixed-size chunks: the node-to-lattice distance
            # table is (chunk, nnodes, nlattice), so memory stays bounded
            # whatever the mesh size
            for i in range(0, len(nodes), self.LINEARISE_CHUNK):
                sl = slice(i, i + self.LINEARISE_CHUNK)
                gv = self._nodepts[verts[sl]][:, vo]
                want = np.einsum('lv,evd->eld', sf, gv)      # (ne, nlat, 3)
                have = self._nodepts[nodes[sl] - self._nodeoff]
                ext = np.ptp(gv, axis=1).max(axis=1)[:, None]
                d = np.linalg.norm(have[:, :, None] - want[:, None], axis=3)
                if not np.all(d.min(axis=2) <= lintol*ext):
                    raise ValueError(f'Curved high-order elements (type '
                                     f'{etype}) are not supported: the '
                                     'geometry path is linear')
        return lin[petype], nodes[:, :nv]

    def _read_eles(self, it):
        elenodes = defaultdict(list)
        if self._version == '2.2':
            for _ in range(int(next(it))):
                v = [int(i) for i in next(it).split()]
                etype, ntags = v[1], v[2]
                self._check_type(etype)
                tags, nodes = v[3:3 + ntags], v[3 + ntags:]
                if len(nodes) != self._nnodes(etype):
                    raise ValueError(f'Element {v[0]}: wrong node count')
                elenodes[etype, (tags[0],)].append(nodes)
        else:
            nb, ne = (int(i) for i in next(it).split()[:2])
            count = 0
            for _ in range(nb):
                edim, etag, etype, ecount = (int(j) for j in next(it).split())
                self._check_type(etype)
                nn = self._nnodes(etype)
                pents = self._tagpents[edim, etag]
                for _ in range(ecount):
                    v = [int(i) for i in next(it).split()]
                    elenodes[etype, pents].append(v[1:nn + 1])
                count += ecount
            if count != ne:
                raise ValueError('Invalid element count')
        out = defaultdict(list)
        for (etype, pents), v in elenodes.items():
            lt, nodes = self._linearise(etype, np.array(v, dtype=np.int64))
            out[lt, pents].append(nodes)
        self._elenodes = {k: np.vstack(v) for k, v in out.items()}

    # ---- assembly ------------------------------------------------------------

    def records(self):
        """The native mesh records (nodes, eles, codec, pmap)."""
        off = self._nodeoff
        pbits = {p: 1 << i
                 for i, (_, p) in enumerate(sorted(self._volpents.items()))}

        # Volume elements by native type (ascending Gmsh type number, then
        # physical group tuple), with their tag masks; boundary elements'
        # first-order vertex sets by physical group
        vol = defaultdict(list)
        tagruns = defaultdict(list)
        bnd = defaultdict(list)
        for (etype, pents), nodes in sorted(self._elenodes.items()):
            petype, _ = GMSH_ETYPES[etype]
            nodes = nodes[:, GMSH_VERTEX_ORDER[petype]] - off
            mask = sum(pbits[p] for p in pents if p in pbits)
            if mask:
                vol[petype].append(nodes)
                tagruns[petype].append((mask, len(nodes)))
            else:
                bnd[pents[0]].append(nodes)
        if not vol:
            raise ValueError('No volume elements in mesh')
        if 'pyr' in vol:
            raise NotImplementedError('Pyramids are not supported')

        etypes = sorted(vol, key=CODEC_ETYPE_ORDER.index)
        ndims = _NDIMS[etypes[0]]
        codec = []
        for et in etypes:
            codec.append(f'eles/{et}')
            codec.extend(f'eles/{et}/face/{i}'
                         for i in range(len(face_vertices(et))))
        codec.extend(f'bc/{b}' for b in self._bfacespents)

        eles = {}
        for et in etypes:
            nodes = np.vstack(vol[et])
            nf = len(face_vertices(et))
            a = np.zeros(len(nodes), dtype=ele_dtype(nodes.shape[1], nf))
            a['nodes'] = nodes
            a['faces']['cidx'] = -1
            a['faces']['off'] = -1
            masks, counts = zip(*tagruns[et])
            a['tags'] = np.repeat(np.array(masks, dtype=np.uint64), counts)
            eles[et] = a

        # Pair the volume faces by vertex set
        keys, refs = [], []
        for et in etypes:
            for fi, fv in enumerate(face_vertices(et)):
                fn = np.sort(eles[et]['nodes'][:, fv], axis=1)
                fn = np.pad(fn, ((0, 0), (0, 4 - fn.shape[1])),
                            constant_values=-1)
                keys.append(fn)
                c = codec.index(f'eles/{et}/face/{fi}')
                refs.append(np.stack([np.full(len(fn), c),
                                      np.arange(len(fn))], axis=1))
        keys, refs = np.vstack(keys), np.vstack(refs)
        o = np.lexsort(keys.T[::-1])
        ks, rs = keys[o], refs[o]
        same = np.all(ks[1:] == ks[:-1], axis=1)
        if np.any(same[1:] & same[:-1]):
            raise ValueError('A face is shared by more than two elements')

        cetype = {codec.index(f'eles/{et}/face/{fi}'): (et, fi)
                  for et in etypes for fi in range(len(face_vertices(et)))}

        def setface(a, b):
            et, fi = cetype[int(a[0])]
            eles[et]['faces'][int(a[1]), fi] = (int(b[0]), int(b[1]))

        paired = np.zeros(len(ks), dtype=bool)
        for i in np.flatnonzero(same):
            setface(rs[i], rs[i + 1])
            setface(rs[i + 1], rs[i])
            paired[i] = paired[i + 1] = True
        resid = {tuple(k[k >= 0].tolist()): tuple(r.tolist())
                 for k, r in zip(ks[~paired], rs[~paired])}

        # Periodic faces
        pmap = {}
        for k, (lp, rp) in self._pfacespents.items():
            plist = []
            lb, rb = bnd.get(lp, []), bnd.get(rp, [])
            ltypes = {x.shape[1] for x in lb}
            for nv in sorted(ltypes):
                lf = np.vstack([x for x in lb if x.shape[1] == nv])
                rf = np.vstack([x for x in rb if x.shape[1] == nv])
                if len(lf) != len(rf):
                    raise ValueError(f'Periodic boundary {k} does not pair')
                lc = self._nodepts[lf][:, :, :ndims].mean(axis=1)
                rc = self._nodepts[rf][:, :, :ndims].mean(axis=1)
                lo_ = fuzzy_lexsort(lc.T, range(len(lf)))
                ro_ = fuzzy_lexsort(rc.T, range(len(rf)))
                for a, b in zip(lf[lo_], rf[ro_]):
                    la = resid.pop(tuple(sorted(a.tolist())))
                    rb_ = resid.pop(tuple(sorted(b.tolist())))
                    setface(la, rb_)
                    setface(rb_, la)
                    plist.append([la, rb_])
            pmap[k] = np.array([[tuple(x) for x in p] for p in plist],
                               dtype=FACE_DTYPE).reshape(-1, 2)

        # Boundary faces
        for name, pent in self._bfacespents.items():
            c = codec.index(f'bc/{name}')
            for fn in bnd.get(pent, []):
                for f in fn:
                    la = resid.pop(tuple(sorted(f.tolist())))
                    et, fi = cetype[la[0]]
                    eles[et]['faces'][la[1], fi] = (c, -1)

        if resid:
            raise ValueError('Unpaired faces in mesh')

        codec.extend(f'tag/{t}' for t in sorted(self._volpents))
        nodes = self._nodepts[:, :ndims].copy()
        return nodes, eles, codec, pmap

    def write(self, fname):
        """Write the native mesh file; returns its identifier."""
        return write_mesh(fname, *self.records())


def import_mesh(msh, fname):
    """Convert a Gmsh file to a native mesh file (``pyfr import``)."""
    return GmshReader(msh).write(fname)
