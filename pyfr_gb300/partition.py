"""Element partitions of a mesh and their interfaces across partitions.

The reference partitions a mesh into one part per MPI rank; each part
holds its elements, the interior interfaces between its own elements, its
boundary faces and, per neighbouring part, the faces it shares with it
(``con_p``, pyfr/readers/native.py:15-47 and pyfr/solvers/base/
system.py:256-263).  Both parts of a shared interface list its faces in the
same order, so that the face data one part packs lines up with the data the
other part receives (pyfr/solvers/baseadvec/inters.py:31-47).

Here the parts are slabs of element centroids along one axis (balanced by
element count), which is what a structured box needs; ``partition`` takes
any conforming mesh.  The part meshes carry ``rank``, ``con_p`` (peer ->
Side) and ``gidx`` (element type -> global indices of the local elements,
ascending) for gathering results back.
"""

import numpy as np

from pyfr_gb300.mesh import Mesh, Side


def _centroids(mesh):
    return {et: sp.mean(axis=0) for et, sp in mesh.spts.items()}


def assign_parts(mesh, nparts, axis=0):
    """Part number of every element: the elements sorted by their
    centroid's coordinate ``axis`` (then by type and index) and cut into
    nparts runs of (nearly) equal size."""
    cen = _centroids(mesh)
    keys = [(c[:, axis], np.full(len(c), i), np.arange(len(c)))
            for i, c in enumerate(cen.values())]
    x = np.concatenate([k[0] for k in keys])
    t = np.concatenate([k[1] for k in keys])
    e = np.concatenate([k[2] for k in keys])
    o = np.lexsort((e, t, x))
    part = np.empty(len(x), dtype=np.int64)
    part[o] = (np.arange(len(x))*nparts)//len(x)
    out, off = {}, 0
    for et, c in cen.items():
        out[et] = part[off:off + len(c)]
        off += len(c)
    return out


def partition(mesh, nparts, axis=0, parts=None):
    """The nparts part meshes of ``mesh`` (element assignment ``parts``,
    by default ``assign_parts(mesh, nparts, axis)``)."""
    parts = parts or assign_parts(mesh, nparts, axis)
    etypes = list(mesh.spts)

    # Global -> local element numbers per part
    gidx = [{et: np.flatnonzero(parts[et] == p) for et in etypes}
            for p in range(nparts)]
    lidx = {et: np.empty(len(parts[et]), dtype=np.int64) for et in etypes}
    for p in range(nparts):
        for et in etypes:
            lidx[et][gidx[p][et]] = np.arange(len(gidx[p][et]))

    def side_arrays(side):
        t = np.asarray(side.etypes)
        e = np.asarray(side.eidxs)
        pp = np.empty(len(e), dtype=np.int64)
        le = np.empty(len(e), dtype=np.int64)
        for et in set(t.tolist()):
            m = t == et
            pp[m] = parts[et][e[m]]
            le[m] = lidx[et][e[m]]
        return t, pp, le, np.asarray(side.fidxs)

    lhs, rhs = mesh.con
    lt, lp, le, lf = side_arrays(lhs)
    rt, rp, re, rf = side_arrays(rhs)

    out = []
    for p in range(nparts):
        inner = (lp == p) & (rp == p)
        con = (Side(lt[inner], le[inner], lf[inner]),
               Side(rt[inner], re[inner], rf[inner]))

        # Faces shared with each peer, in the global interface order
        con_p = {}
        for q in range(nparts):
            if q == p:
                continue
            a = (lp == p) & (rp == q)
            b = (rp == p) & (lp == q)
            k = np.flatnonzero(a | b)
            if not len(k):
                continue
            mine_l = a[k]
            t = np.where(mine_l, lt[k], rt[k])
            e = np.where(mine_l, le[k], re[k])
            f = np.where(mine_l, lf[k], rf[k])
            con_p[q] = Side(t, e, f)

        bcon = {}
        for name, side in getattr(mesh, 'bcon', {}).items():
            bt, bp, be, bf = side_arrays(side)
            m = bp == p
            if m.any():
                bcon[name] = Side(bt[m], be[m], bf[m])

        spts = {et: mesh.spts[et][:, gidx[p][et]] for et in etypes
                if len(gidx[p][et])}
        curved = {et: mesh.spts_curved.get(
            et, np.zeros(len(parts[et]), dtype=bool))[gidx[p][et]]
            for et in spts}
        pm = Mesh(ndims=mesh.ndims, spts=spts, con=con, spts_curved=curved,
                  periods=mesh.periods, bcon=bcon)
        pm.rank, pm.nparts = p, nparts
        pm.con_p = con_p
        pm.gidx = {et: gidx[p][et] for et in spts}
        out.append(pm)
    return out


def gather_field(parts, fields, nglobal):
    """Assemble per-part element fields ({etype: (..., neles_local)}) into
    global arrays ({etype: (..., nglobal[etype])})."""
    out = {}
    for pm, f in zip(parts, fields):
        for et, a in f.items():
            g = out.setdefault(et, np.zeros(a.shape[:-1] + (nglobal[et],),
                                            dtype=a.dtype))
            g[..., pm.gidx[et]] = a
    return out
