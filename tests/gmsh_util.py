"""Writers of small ASCII Gmsh files for the mesh-import tests (test
infrastructure): structured boxes of quadrilaterals or hexahedra with named
volume, boundary and periodic physical groups, in the 2.2 and 4.1 formats."""
import numpy as np

# Gmsh vertex order of a quad / hex from the first-coordinate-fastest order
_TO_GMSH = {2: [0, 1, 3, 2], 3: [0, 1, 3, 2, 4, 5, 7, 6]}


def box_msh(n, periodic, version='2.2', lo=0.0, hi=1.0, vol='fluid'):
    """Gmsh text of a box of n[0] x n[1] (x n[2]) cells on [lo, hi]^d.

    Cells are numbered x fastest.  A periodic direction d has the physical
    groups periodic_<d>_l / periodic_<d>_r on its low / high faces; a
    bounded one has the boundaries '<x|y|z>lo' / '<x|y|z>hi'."""
    nd = len(n)
    axes = [np.linspace(lo, hi, k + 1) for k in n]
    shape = [k + 1 for k in n]
    nid = np.arange(1, np.prod(shape) + 1).reshape(shape[::-1])  # [z][y][x]

    def node(ijk):
        return int(nid[tuple(ijk[::-1])])

    nodes = []
    for ijk in np.ndindex(*shape[::-1]):
        ijk = ijk[::-1]
        nodes.append((node(ijk), [float(axes[d][ijk[d]]) for d in range(nd)]
                      + [0.0]*(3 - nd)))

    # Volume elements
    cells = []
    for ijk in np.ndindex(*n[::-1]):
        ijk = ijk[::-1]
        vs = [node([ijk[d] + ((v >> d) & 1) for d in range(nd)])
              for v in range(2**nd)]
        cells.append([vs[i] for i in _TO_GMSH[nd]])

    # Boundary facets of each side: (physical name, list of facets)
    groups = []
    for d in range(nd):
        for side, name in ((0, 'l'), (1, 'r')):
            pname = (f'periodic_{d}_{name}' if periodic[d] else
                     f'{"xyz"[d]}{"lo" if side == 0 else "hi"}')
            facets = []
            others = [e for e in range(nd) if e != d]
            for idx in np.ndindex(*[n[e] for e in others][::-1]):
                idx = idx[::-1]
                corners = []
                for v in range(2**(nd - 1)):
                    ijk = [0]*nd
                    ijk[d] = side*n[d]
                    for k, e in enumerate(others):
                        ijk[e] = idx[k] + ((v >> k) & 1)
                    corners.append(node(ijk))
                if nd == 3:
                    corners = [corners[i] for i in (0, 1, 3, 2)]
                facets.append(corners)
            groups.append((pname, facets))

    ftype = {2: 1, 3: 3}[nd]
    vtype = {2: 3, 3: 5}[nd]
    names = [(nd, 1, vol)] + [(nd - 1, 2 + i, g[0])
                              for i, g in enumerate(groups)]
    out = ['$MeshFormat', f'{version} 0 8', '$EndMeshFormat',
           '$PhysicalNames', str(len(names))]
    out += [f'{d} {t} "{nm}"' for d, t, nm in names]
    out.append('$EndPhysicalNames')

    if version == '2.2':
        out += ['$Nodes', str(len(nodes))]
        out += [f'{i} {x[0]!r} {x[1]!r} {x[2]!r}' for i, x in nodes]
        out += ['$EndNodes', '$Elements']
        els = [(ftype, 2 + gi, f) for gi, (_, fs) in enumerate(groups)
               for f in fs]
        els += [(vtype, 1, c) for c in cells]
        out.append(str(len(els)))
        out += [f'{k + 1} {t} 2 {p} {p} ' + ' '.join(map(str, v))
                for k, (t, p, v) in enumerate(els)]
        out.append('$EndElements')
    else:
        # One entity per physical group: surfaces/curves for the facets
        # and one volume (surface in 2-D)
        ents = [0, 0, 0]
        lines = []
        fdim = nd - 1
        ents[fdim - 1] = len(groups)
        ents[nd - 1] = 1
        for gi in range(len(groups)):
            lines.append(f'{gi + 1} 0 0 0 1 1 1 1 {2 + gi} 0')
        lines.append('1 0 0 0 1 1 1 1 1 0')
        out += ['$Entities', f'0 {ents[0]} {ents[1]} {ents[2]}'] + lines
        out.append('$EndEntities')
        out += ['$Nodes', f'1 {len(nodes)} 1 {len(nodes)}',
                f'{nd} 1 0 {len(nodes)}']
        out += [str(i) for i, _ in nodes]
        out += [f'{x[0]!r} {x[1]!r} {x[2]!r}' for _, x in nodes]
        out.append('$EndNodes')
        nel = sum(len(f) for _, f in groups) + len(cells)
        out += ['$Elements', f'{len(groups) + 1} {nel} 1 {nel}']
        k = 1
        for gi, (_, fs) in enumerate(groups):
            out.append(f'{fdim} {gi + 1} {ftype} {len(fs)}')
            for f in fs:
                out.append(f'{k} ' + ' '.join(map(str, f)))
                k += 1
        out.append(f'{nd} 1 {vtype} {len(cells)}')
        for c in cells:
            out.append(f'{k} ' + ' '.join(map(str, c)))
            k += 1
        out.append('$EndElements')
    return '\n'.join(out) + '\n'


def raise_order(txt, order, perturb=None):
    """A version-2.2 Gmsh text of straight elements of ``order`` from the
    first-order text of ``box_msh``: each quadrilateral and hexahedron
    gets the nodes of the equi-spaced lattice of its vertices after them
    (the importer matches nodes to lattice points whatever their order).
    ``perturb``: (element number, lattice node index, offset) moves one
    added node off the lattice."""
    hexq = {3: (10, 36, 37), 5: (12, 92, 93)}        # linear -> order 2-4
    inv = {2: [0, 1, 3, 2], 3: [0, 1, 3, 2, 4, 5, 7, 6]}
    lines = txt.split('\n')
    i0, i1 = lines.index('$Nodes'), lines.index('$EndNodes')
    pts = {}
    for ln in lines[i0 + 2:i1]:
        v = ln.split()
        pts[int(v[0])] = np.array([float(x) for x in v[1:4]])
    nxt = max(pts) + 1
    e0, e1 = lines.index('$Elements'), lines.index('$EndElements')
    els, new = [], []
    for ln in lines[e0 + 2:e1]:
        v = [int(x) for x in ln.split()]
        num, et, nt = v[0], v[1], v[2]
        vs = v[3 + nt:]
        if et not in hexq:
            els.append(ln)
            continue
        nd = 2 if et == 3 else 3
        # Vertices in first-coordinate-fastest order
        corner = np.array([pts[vs[inv[nd].index(k)]] for k in range(2**nd)])
        extra = []
        for ijk in np.ndindex(*(order + 1,)*nd):
            t = np.array(ijk[::-1], dtype=float)/order
            if np.all((t == 0) | (t == 1)):
                continue
            w = np.ones(2**nd)
            for k in range(2**nd):
                for d in range(nd):
                    w[k] *= t[d] if (k >> d) & 1 else 1 - t[d]
            x = w @ corner
            if perturb and perturb[0] == num and perturb[1] == len(extra):
                x = x + np.asarray(perturb[2])
            pts[nxt] = x
            new.append(nxt)
            extra.append(nxt)
            nxt += 1
        ht = hexq[et][order - 2]
        els.append(' '.join(map(str, [num, ht, nt, *v[3:3 + nt], *vs,
                                      *extra])))
    nodes = [f'{k} {float(x[0])!r} {float(x[1])!r} {float(x[2])!r}'
             for k, x in sorted(pts.items())]
    out = lines[:i0 + 1] + [str(len(nodes))] + nodes + lines[i1:e0 + 1]
    out += [str(len(els))] + els + lines[e1:]
    return '\n'.join(out)
