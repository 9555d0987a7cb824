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

    @property
    def etypes(self):
        return list(self.spts)


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
