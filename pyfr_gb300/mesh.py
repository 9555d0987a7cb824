"""Synthetic meshes and interface connectivity.

A mesh carries, per element type, the shape points (``spts``, io-shape
(nspts, neles, ndims), vertex order first-coordinate-fastest) and the
interior interfaces as two aligned sides (lhs, rhs) of
(element type, element index, face index) triples.  This is the content
of the reference's ``Mesh``/``Connectivity`` (``pyfr/readers/native.py:15-86``)
that the right-hand side needs; meshes are generated here instead of being
read from HDF5.
"""

from dataclasses import dataclass, field

import numpy as np


class Side:
    """One side of a set of interfaces (the reference's Connectivity)."""

    def __init__(self, etypes, eidxs, fidxs):
        self.etypes = np.asarray(etypes)
        self.eidxs = np.asarray(eidxs, dtype=np.int64)
        self.fidxs = np.asarray(fidxs, dtype=np.int64)

    def __len__(self):
        return len(self.eidxs)

    def _groups(self):
        keys = sorted(set(zip(self.etypes.tolist(), self.fidxs.tolist())))
        for et, fi in keys:
            mask = (self.etypes == et) & (self.fidxs == fi)
            yield et, fi, mask

    def items(self):
        for et, fi, mask in self._groups():
            yield et, fi, self.eidxs[mask]

    def foreach(self):
        for et, fi, mask in self._groups():
            yield et, fi, self.eidxs[mask], np.flatnonzero(mask)


@dataclass
class Mesh:
    ndims: int
    spts: dict
    con: tuple
    spts_curved: dict = field(default_factory=dict)
    periods: tuple = None
    # Boundary faces by boundary name: Side of (etype, element, face)
    # (the reference's bcon_<name> arrays, pyfr/readers/native.py:15-86)
    bcon: dict = field(default_factory=dict)
    # Records of a mesh read from a file: its identifier, codec, the file's
    # numbers of the elements of each type (local order), and so on
    uuid: str = None
    codec: list = None
    eidxs: dict = None
    fname: str = None
    creator: str = None
    colours: dict = None
    tags: dict = None
    spts_nodes: dict = None

    @property
    def etypes(self):
        return list(self.spts)


def vertex_nodes(mesh, tol=1e-9):
    """Global node numbers of the vertices of every element: per element
    type an array (nverts, neles), and the number of nodes.  A mesh read
    from a file numbers them by its node table (``spts_nodes``); otherwise
    coincident vertices (within ``tol`` of the mesh extent) share a node,
    numbered by first appearance over the types in ``spts`` order.  As in
    a mesh file, the two sides of a periodic boundary have distinct
    nodes."""
    if mesh.spts_nodes:
        from pyfr_gb300.native import corner_nodes, _order_from_nnodes
        from pyfr_gb300.shapes import VERTICES
        out = {}
        for et, sn in mesh.spts_nodes.items():
            nn = sn.shape[1]
            cn = list(range(nn)) if nn == len(VERTICES[et]) else \
                corner_nodes(et, _order_from_nnodes(et, nn))
            out[et] = sn[:, cn].T
        allv = np.concatenate([v.ravel() for v in out.values()])
        uniq, inv = np.unique(allv, return_inverse=True)
        off = 0
        for et, v in out.items():
            out[et] = inv[off:off + v.size].reshape(v.shape)
            off += v.size
        return out, len(uniq)

    etypes = list(mesh.spts)
    allpts = np.concatenate([mesh.spts[et].reshape(-1, mesh.ndims)
                             for et in etypes])
    scale = max(np.ptp(allpts, axis=0).max(), 1.0)
    q = np.rint(allpts / (tol*scale)).astype(np.int64)
    _, first, inv = np.unique(q, axis=0, return_index=True,
                              return_inverse=True)
    remap = np.empty(len(first), dtype=np.int64)
    remap[np.argsort(first)] = np.arange(len(first))
    nid = remap[inv.ravel()]
    out, off = {}, 0
    for et in etypes:
        nv, ne = mesh.spts[et].shape[:2]
        out[et] = nid[off:off + nv*ne].reshape(nv, ne)
        off += nv*ne
    return out, len(first)


def periodic_box(etype, ncells, lo, hi):
    """Uniform periodic box of quads (2-D) or hexes (3-D).

    ``ncells`` cells per direction (int or tuple), domain [lo, hi]^ndims.
    Element index i + n0*(j + n1*k); every face is an interior interface
    (the +x/+y/+z face of a cell is the left side).
    """
    ndims = {'quad': 2, 'hex': 3}[etype]
    n = (ncells,)*ndims if np.isscalar(ncells) else tuple(ncells)
    lo = (lo,)*ndims if np.isscalar(lo) else tuple(lo)
    hi = (hi,)*ndims if np.isscalar(hi) else tuple(hi)

    axes = [np.linspace(lo[d], hi[d], n[d] + 1) for d in range(ndims)]
    idx = np.indices(n[::-1]).reshape(ndims, -1)[::-1]      # (ndims, neles)
    neles = idx.shape[1]

    # Vertices in first-coordinate-fastest order
    nverts = 2**ndims
    spts = np.empty((nverts, neles, ndims))
    for v in range(nverts):
        for d in range(ndims):
            off = (v >> d) & 1
            spts[v, :, d] = axes[d][idx[d] + off]

    def eid(ijk):
        e = np.zeros(neles, dtype=np.int64)
        stride = 1
        for d in range(ndims):
            e += (ijk[d] % n[d])*stride
            stride *= n[d]
        return e

    # (left face, right face) of a neighbour pair across each axis
    facepairs = {'quad': [(1, 3), (2, 0)],
                 'hex': [(2, 4), (3, 1), (5, 0)]}[etype]

    lt, le, lf, rt, re, rf = [], [], [], [], [], []
    here = eid(idx)
    for d, (fl, fr) in enumerate(facepairs):
        nb = idx.copy()
        nb[d] += 1
        le.append(here)
        lf.append(np.full(neles, fl))
        re.append(eid(nb))
        rf.append(np.full(neles, fr))

    lhs = Side([etype]*neles*ndims, np.concatenate(le), np.concatenate(lf))
    rhs = Side([etype]*neles*ndims, np.concatenate(re), np.concatenate(rf))

    periods = tuple(hi[d] - lo[d] for d in range(ndims))
    return Mesh(ndims=ndims, spts={etype: spts}, con=(lhs, rhs),
                spts_curved={etype: np.zeros(neles, dtype=bool)},
                periods=periods)


def box(etype, ncells, lo, hi, periodic, bcnames=None):
    """Uniform box of quads (2-D) or hexes (3-D), periodic in the directions
    flagged in ``periodic`` and bounded in the others.  The faces at the
    low and high ends of a bounded direction d form the boundaries named
    ``bcnames[d] = (low name, high name)`` (default 'xlo'/'xhi' and so on).
    Elements are numbered x fastest."""
    ndims = {'quad': 2, 'hex': 3}[etype]
    n = (ncells,)*ndims if np.isscalar(ncells) else tuple(ncells)
    lo = (lo,)*ndims if np.isscalar(lo) else tuple(lo)
    hi = (hi,)*ndims if np.isscalar(hi) else tuple(hi)
    periodic = tuple(periodic)

    axes = [np.linspace(lo[d], hi[d], n[d] + 1) for d in range(ndims)]
    idx = np.indices(n[::-1]).reshape(ndims, -1)[::-1]
    neles = idx.shape[1]
    spts = np.empty((2**ndims, neles, ndims))
    for v in range(2**ndims):
        for d in range(ndims):
            spts[v, :, d] = axes[d][idx[d] + ((v >> d) & 1)]

    def eid(ijk):
        e = np.zeros(ijk.shape[1], dtype=np.int64)
        stride = 1
        for d in range(ndims):
            e += (ijk[d] % n[d])*stride
            stride *= n[d]
        return e

    # (face at the high end, face at the low end) of each direction
    facepairs = {'quad': [(1, 3), (2, 0)],
                 'hex': [(2, 4), (3, 1), (5, 0)]}[etype]
    names = bcnames or [(f'{a}lo', f'{a}hi') for a in 'xyz'[:ndims]]
    le, lf, re, rf = [], [], [], []
    bcon = {}
    here = eid(idx)
    for d, (fhi, flo) in enumerate(facepairs):
        inner = np.ones(neles, dtype=bool) if periodic[d] else \
            idx[d] < n[d] - 1
        nb = idx.copy()
        nb[d] += 1
        le.append(here[inner])
        lf.append(np.full(inner.sum(), fhi))
        re.append(eid(nb[:, inner]))
        rf.append(np.full(inner.sum(), flo))
        if not periodic[d]:
            for name, sel, f in ((names[d][0], idx[d] == 0, flo),
                                 (names[d][1], idx[d] == n[d] - 1, fhi)):
                e = here[sel]
                prev = bcon.get(name)
                sd = Side([etype]*len(e), e, np.full(len(e), f))
                if prev is not None:
                    sd = Side(np.concatenate([prev.etypes, sd.etypes]),
                              np.concatenate([prev.eidxs, sd.eidxs]),
                              np.concatenate([prev.fidxs, sd.fidxs]))
                bcon[name] = sd

    nint = sum(len(x) for x in le)
    lhs = Side([etype]*nint, np.concatenate(le), np.concatenate(lf))
    rhs = Side([etype]*nint, np.concatenate(re), np.concatenate(rf))
    periods = tuple((hi[d] - lo[d]) if periodic[d] else None
                    for d in range(ndims))
    return Mesh(ndims=ndims, spts={etype: spts}, con=(lhs, rhs),
                spts_curved={etype: np.zeros(neles, dtype=bool)},
                periods=periods, bcon=bcon)


def face_vertices(etype):
    """Vertex indices of each face of a linear ``etype`` element, in the
    reference's face order (from the face projections of the shape)."""
    from pyfr_gb300.shapes import SHAPES, VERTICES

    corners = {'line': [(-1,), (1,)], 'tri': [(-1, -1), (1, -1), (-1, 1)],
               'quad': [(-1, -1), (1, -1), (-1, 1), (1, 1)]}
    verts = np.array(VERTICES[etype], dtype=float)
    out = []
    for kind, proj, norm in SHAPES[etype].faces:
        fv = []
        for c in corners[kind]:
            x = np.array(proj(*c), dtype=float)
            (i,) = np.flatnonzero(np.all(np.abs(verts - x) < 1e-12, axis=1))
            fv.append(int(i))
        out.append(fv)
    return out


def connect(spts, periods=None, lo=None, tol=1e-8):
    """Interior interfaces of a conforming mesh: faces of linear elements
    paired by their centroids (reduced modulo ``periods`` measured from
    ``lo``) and their vertex offsets from the centroid, so that a periodic
    box of any size pairs unambiguously.  ``spts`` maps element types to
    their vertices (nverts, neles, ndims).  Every face must pair up (no
    boundaries).  Returns the (lhs, rhs) sides; of the two faces of an
    interface the one met first (types in ``spts`` order, then element,
    then face) is the left one."""
    keys, ids = [], []
    for et, sp in spts.items():
        ndims = sp.shape[2]
        for fi, fv in enumerate(face_vertices(et)):
            c = sp[fv]                                 # (nfv, neles, ndims)
            cen = c.mean(axis=0)
            rel = np.rint((c - cen)/tol).astype(np.int64)
            if periods is not None:
                per = np.asarray(periods, dtype=float)
                cen = np.mod(cen - np.asarray(lo, dtype=float), per)
                cen[np.abs(cen - per) < tol*per] = 0.0
            qc = np.rint(cen/tol).astype(np.int64)     # (neles, ndims)

            # Order the face's vertices to make the key orientation-free
            rel = rel.transpose(1, 0, 2)               # (neles, nfv, ndims)
            o = np.lexsort(tuple(rel[:, :, d]
                                 for d in reversed(range(ndims))), axis=1)
            rel = np.take_along_axis(rel, o[:, :, None], axis=1)
            keys.append(np.hstack([qc, rel.reshape(rel.shape[0], -1)]))
            ids.append(np.stack([np.full(len(qc), list(spts).index(et)),
                                 np.arange(len(qc)), np.full(len(qc), fi)],
                                1))

    nk = max(k.shape[1] for k in keys)
    keys = np.vstack([np.pad(k, ((0, 0), (0, nk - k.shape[1])),
                             constant_values=-1) for k in keys])
    ids = np.vstack(ids)
    order = np.lexsort(keys.T[::-1])
    ks = keys[order]
    same = np.all(ks[1:] == ks[:-1], axis=1)
    if len(ks) % 2 or not np.all(same[::2]) or np.any(same[1::2]):
        raise ValueError('Mesh faces do not pair up into interfaces')
    a, b = ids[order[0::2]], ids[order[1::2]]

    # Left side: the earlier face
    swap = (a[:, 0]*2**40 + a[:, 1]*8 + a[:, 2]) > \
        (b[:, 0]*2**40 + b[:, 1]*8 + b[:, 2])
    a[swap], b[swap] = b[swap], a[swap].copy()
    o = np.lexsort((a[:, 2], a[:, 1], a[:, 0]))
    a, b = a[o], b[o]
    names = np.array(list(spts))
    return (Side(names[a[:, 0]], a[:, 1], a[:, 2]),
            Side(names[b[:, 0]], b[:, 1], b[:, 2]))


def _cube_cells(n, lo, hi):
    """Cell corner coordinates of a uniform n^3 grid: (8, ncells, 3) with
    corners in first-coordinate-fastest order, and the cell indices."""
    axes = [np.linspace(lo, hi, n + 1)]*3
    idx = np.indices((n, n, n)).reshape(3, -1)[::-1]       # i fastest
    c = np.empty((8, idx.shape[1], 3))
    for v in range(8):
        for d in range(3):
            c[v, :, d] = axes[d][idx[d] + ((v >> d) & 1)]
    return c, idx


# Corners (first-coordinate-fastest numbering of the cube) of the two
# prisms of a cube cut along the diagonal plane through its (0,0)-(1,1)
# edge pairs, each with the right-angle vertex first and positive volume
_PRI_OF_CUBE = [[1, 3, 0, 5, 7, 4], [2, 0, 3, 6, 4, 7]]


def _tets_of_cube():
    """Corners of the six tetrahedra of the cube's Kuhn subdivision (one
    per path (0,0,0) -> (1,1,1) along the axes), in the reference's vertex
    order with positive volume.  All cubes cut this way conform, and each
    of their z faces is cut along the same diagonal as the prisms'."""
    out = []
    for perm in [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1),
                 (2, 1, 0)]:
        path, v = [0], 0
        for d in perm:
            v |= 1 << d
            path.append(v)
        pts = np.array([[(c >> d) & 1 for d in range(3)] for c in path], float)
        if np.linalg.det((pts[1:] - pts[0]).T) < 0:
            path[1], path[2] = path[2], path[1]
        out.append(path)
    return out


def _orient(v, ref):
    """Swap vertices ref[1] and ref[2] of the elements (v: (nverts, neles,
    3)) whose frame (v[r1] - v[r0]) x (v[r2] - v[r0]) . (v[r3] - v[r0]) is
    negative, ref = (r0, r1, r2, r3)."""
    r0, r1, r2, r3 = ref
    a, b, c = v[r1] - v[r0], v[r2] - v[r0], v[r3] - v[r0]
    neg = np.einsum('ei,ei->e', np.cross(a, b), c) < 0
    t = v[r1, neg].copy()
    v[r1, neg] = v[r2, neg]
    v[r2, neg] = t
    return v


def _pyr_tet_cells(corners, idx, sel, n, cut=True):
    """The cells ``sel`` cut into six pyramids, one on each face with its
    apex at the cell centre; the pyramid on a face shared with a hex cell
    (x index below n/2) is kept, every other one (with ``cut``) is cut
    into two tetrahedra along the face diagonal through the face's corners
    of even in-plane lattice parity, which the cell across the face (and a
    periodic image) cuts the same way.  Returns pyramid and tetrahedron
    vertices (nverts, neles, 3)."""
    cen = corners[:, sel].mean(axis=0)
    ci = idx[:, sel]
    pyrs, tets = [], []
    for a in range(3):
        u, v = [d for d in range(3) if d != a]
        for side in (0, 1):
            # Face corners in tensor order (u fastest), cube numbering
            # first-coordinate-fastest
            fc = [(side << a) | (bu << u) | (bv << v)
                  for bv in (0, 1) for bu in (0, 1)]
            base = corners[fc][:, sel]                   # (4, ncell, 3)
            if not cut:
                keep = np.ones(ci.shape[1], dtype=bool)
            elif a == 0:
                nb = (ci[0] + (1 if side else -1)) % n
                keep = nb < n//2
            else:
                keep = np.zeros(ci.shape[1], dtype=bool)
            if keep.any():
                pv = np.concatenate([base[:, keep], cen[None, keep]])
                pyrs.append(_orient(pv, (0, 1, 2, 4)))
            cut_here = ~keep
            if not cut_here.any():
                continue
            even = ((ci[u] + ci[v]) % 2 == 0)[cut_here]
            b, c = base[:, cut_here], cen[cut_here]
            # Diagonal (0, 3) where the corner 0 has even parity, else (1, 2)
            d0 = np.where(even[:, None], b[0], b[1])
            d1 = np.where(even[:, None], b[3], b[2])
            o1 = np.where(even[:, None], b[1], b[0])
            o2 = np.where(even[:, None], b[2], b[3])
            for o in (o1, o2):
                tv = np.stack([d0, d1, o, c])
                tets.append(_orient(tv, (0, 1, 2, 3)))
    return (np.concatenate(pyrs, axis=1),
            np.concatenate(tets, axis=1) if tets else None)


def mixed_box(n, lo, hi, kinds):
    """Conforming periodic box of n^3 cubic cells of side (hi - lo)/n.

    ``kinds`` is 'hex-pri' (cells with x index below n/2 are hexes, the
    others are cut into two prisms extruded along z), 'pri-tet' (cells
    with z index below n/2 are cut into two prisms, the others into the six
    tetrahedra of the Kuhn subdivision) or 'hex-pyr-tet' (cells with x
    index below n/2 are hexes; the others are cut into six pyramids about
    their centres, and every pyramid whose base is not shared with a hex
    into two tetrahedra, so that hexes and tetrahedra meet through
    pyramids) or 'pyr' (every cell cut into its six pyramids).  A hex face
    never meets a tetrahedron: their quadrilateral and triangular faces do
    not conform.  Elements of each type are numbered cell by cell, x
    fastest, except in 'hex-pyr-tet' and 'pyr', where the pyramids and
    tetrahedra are numbered face by face."""
    corners, idx = _cube_cells(n, lo, hi)
    if kinds in ('hex-pyr-tet', 'pyr'):
        if n < 2:
            raise ValueError(f'{kinds} needs at least two cells a side')
        if kinds == 'pyr':
            pyr, _ = _pyr_tet_cells(corners, idx,
                                    np.ones(idx.shape[1], dtype=bool), n,
                                    cut=False)
            spts = {'pyr': pyr}
        else:
            first = idx[0] < n//2
            pyr, tet = _pyr_tet_cells(corners, idx, ~first, n)
            spts = {'hex': corners[:, first], 'pyr': pyr, 'tet': tet}
        con = connect(spts, periods=(hi - lo,)*3, lo=(lo,)*3)
        return Mesh(ndims=3, spts=spts, con=con,
                    spts_curved={k: np.zeros(v.shape[1], dtype=bool)
                                 for k, v in spts.items()},
                    periods=(hi - lo,)*3)
    if kinds == 'hex-pri':
        first = idx[0] < n//2
        spts = {'hex': corners[:, first],
                'pri': np.stack([corners[c][:, ~first]
                                 for c in _PRI_OF_CUBE], axis=2)}
    elif kinds == 'pri-tet':
        first = idx[2] < n//2
        spts = {'pri': np.stack([corners[c][:, first]
                                 for c in _PRI_OF_CUBE], axis=2),
                'tet': np.stack([corners[c][:, ~first]
                                 for c in _tets_of_cube()], axis=2)}
    else:
        raise ValueError(f'Unknown mixed mesh {kinds!r}')

    # (nverts, ncells, nsub, 3) -> (nverts, ncells*nsub, 3), cell major
    spts = {k: v.reshape(v.shape[0], -1, 3) for k, v in spts.items()}
    con = connect(spts, periods=(hi - lo,)*3, lo=(lo,)*3)
    return Mesh(ndims=3, spts=spts, con=con,
                spts_curved={k: np.zeros(v.shape[1], dtype=bool)
                             for k, v in spts.items()},
                periods=(hi - lo,)*3)


def tri_box(n, lo, hi):
    """Periodic square of n x n cells, each cut into two triangles along its
    (0,0)-(1,1) diagonal (vertices in the reference's order with positive
    area); elements numbered cell by cell, x fastest."""
    axes = np.linspace(lo, hi, n + 1)
    idx = np.indices((n, n)).reshape(2, -1)[::-1]          # i fastest
    corners = np.empty((4, idx.shape[1], 2))
    for v in range(4):
        for d in range(2):
            corners[v, :, d] = axes[idx[d] + ((v >> d) & 1)]
    # corners 0 (0,0), 1 (1,0), 2 (0,1), 3 (1,1): triangles (1,3,0), (2,0,3)
    spts = np.stack([corners[[1, 3, 0]], corners[[2, 0, 3]]], axis=2)
    spts = {'tri': spts.reshape(3, -1, 2)}
    con = connect(spts, periods=(hi - lo,)*2, lo=(lo,)*2)
    return Mesh(ndims=2, spts=spts, con=con,
                spts_curved={'tri': np.zeros(spts['tri'].shape[1], bool)},
                periods=(hi - lo,)*2)


def fuzzy_face_order(coords, tol=1e-6):
    """Per-face ordering of flux points by their physical coordinates,
    lexicographic with the first coordinate most significant and values
    within ``tol`` treated as equal; coords has shape (n, ndims, nfp).

    Both sides of an interface (or the two translated copies of a periodic
    face) sort into the same order, which is what pairs their flux points
    (``pyfr/solvers/base/elements.py:161-172``, ``pyfr/nputil.py:168-183``).
    """
    n, ndims, nfp = coords.shape
    rel = coords - coords.min(axis=2, keepdims=True)
    q = np.rint(rel / tol).astype(np.int64)
    keys = tuple(q[:, d, :] for d in reversed(range(ndims)))
    return np.lexsort(keys, axis=-1)
