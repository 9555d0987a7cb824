"""Point sets and quadrature rules on the reference elements.

The reference element conventions are those of ``pyfr/shapes.py``: the
line and quad/hex span [-1, 1] in every coordinate; the triangle has the
vertices (-1,-1), (1,-1), (-1,1); the tetrahedron (-1,-1,-1), (1,-1,-1),
(-1,1,-1), (-1,-1,1); the prism is the triangle extruded over z in [-1, 1].

Everything here is computed, not tabulated:

* Gauss-Legendre and Gauss-Legendre-Lobatto rules on the line (and their
  tensor products on quads, hexes and, with a triangle rule, prisms);
* collapsed-coordinate (Duffy) Gauss rules on the triangle and the
  tetrahedron, exact for polynomials of a requested total degree; these
  integrate the lifting operators and mass matrices of the simplex shapes,
  where the reference uses tabulated symmetric rules of at least the same
  degree (``pyfr/shapes.py:232-255``) -- exact rules give the same
  integrals up to rounding;
* the collapsed Gauss rule of the pyramid and its layered Gauss-Legendre
  and Gauss-Legendre-Lobatto point sets (``pyfr/quadrules/pyr``);
* the warp-and-blend 'alpha-optimised' interpolation nodes on the triangle
  and tetrahedron (T. Warburton, J. Eng. Math. 56, 2006, 247-262; the
  optimised blending parameters are the ones published there), the point
  sets the reference names ``alpha-opt`` (``pyfr/quadrules/tri``,
  ``pyfr/quadrules/tet``; both use the tetrahedron's parameters).  The points here are listed in the order of the
  equispaced lattice they are warped from (x fastest, then y, then z),
  which for the tetrahedron is also the order of the reference's table;
  the reference's triangle table lists the same points grouped by symmetry
  orbit instead.

A rule may also be given literally, in the reference's text format for
tabulated rules (``pyfr/quadrules/__init__.py:7-40``): one point per line
(or parenthesised tuples), coordinates optionally followed by a weight.
"""

import itertools as it
import math
import re

import numpy as np


# ---------------------------------------------------------------------------
# Line rules
# ---------------------------------------------------------------------------

def gauss_legendre(n):
    """n-point Gauss-Legendre rule on [-1, 1] (ascending abscissae)."""
    return np.polynomial.legendre.leggauss(n)


def gauss_legendre_lobatto(n):
    """n-point Gauss-Legendre-Lobatto rule on [-1, 1]."""
    if n < 2:
        raise ValueError('Lobatto rules need at least two points')

    # Interior nodes are the roots of P'_{n-1}
    c = np.zeros(n)
    c[-1] = 1
    inner = np.polynomial.legendre.legroots(np.polynomial.legendre.legder(c))
    x = np.concatenate([[-1.0], np.sort(inner.real), [1.0]])
    pn1 = np.polynomial.legendre.legval(x, c)
    w = 2.0 / (n*(n - 1)*pn1**2)
    return x, w


RULES_1D = {
    'gauss-legendre': gauss_legendre,
    'gauss-legendre-lobatto': gauss_legendre_lobatto,
}


def tensor_rule(name, n1d, ndims):
    """Tensor-product rule with the first coordinate varying fastest, the
    ordering of the tabulated rules in ``pyfr/quadrules/{quad,hex}``."""
    x, w = RULES_1D[name](n1d)
    pts = np.array([p[::-1] for p in it.product(x, repeat=ndims)])
    wts = np.array([np.prod(q) for q in it.product(w, repeat=ndims)])
    return pts.reshape(-1, ndims), wts


# ---------------------------------------------------------------------------
# Collapsed Gauss rules on simplices
# ---------------------------------------------------------------------------

def tri_gauss(qdeg):
    """Collapsed Gauss-Legendre rule on the reference triangle exact for
    polynomials of total degree ``qdeg``: the square [-1,1]^2 mapped by
    r = (1 + u)(1 - v)/2 - 1, s = v, with Jacobian (1 - v)/2."""
    n = qdeg//2 + 1 + 1
    x, w = gauss_legendre(n)
    u, v = np.meshgrid(x, x, indexing='xy')
    wu, wv = np.meshgrid(w, w, indexing='xy')
    u, v, wu, wv = u.ravel(), v.ravel(), wu.ravel(), wv.ravel()
    pts = np.stack([(1 + u)*(1 - v)/2 - 1, v], axis=1)
    return pts, wu*wv*(1 - v)/2


def tet_gauss(qdeg):
    """Collapsed Gauss-Legendre rule on the reference tetrahedron exact for
    total degree ``qdeg``: r = (1 + u)(1 - v)(1 - w)/4 - 1,
    s = (1 + v)(1 - w)/2 - 1, t = w, Jacobian (1 - v)/2 ((1 - w)/2)^2."""
    n = qdeg//2 + 2
    x, wx = gauss_legendre(n)
    g = np.array(list(it.product(range(n), repeat=3)))
    w_, v, u = x[g[:, 0]], x[g[:, 1]], x[g[:, 2]]
    wts = wx[g[:, 0]]*wx[g[:, 1]]*wx[g[:, 2]]
    pts = np.stack([(1 + u)*(1 - v)*(1 - w_)/4 - 1,
                    (1 + v)*(1 - w_)/2 - 1, w_], axis=1)
    return pts, wts*(1 - v)/2*((1 - w_)/2)**2


def pri_gauss(qdeg):
    """Triangle rule times a Gauss-Legendre line rule in z."""
    tp, tw = tri_gauss(qdeg)
    lp, lw = gauss_legendre(qdeg//2 + 1)
    pts = np.array([[*p, z] for z in lp for p in tp])
    wts = np.array([a*b for b in lw for a in tw])
    return pts, wts


def pyr_gauss(qdeg):
    """Collapsed Gauss-Legendre rule on the reference pyramid (base
    [-1,1]^2 at z = -1, apex (0, 0, 1)) exact for total degree ``qdeg``:
    the cube [-1,1]^3 mapped by x = u(1 - w)/2, y = v(1 - w)/2, z = w,
    whose Jacobian ((1 - w)/2)^2 raises the degree in w by two."""
    n, nz = qdeg//2 + 1, (qdeg + 2)//2 + 1
    x, wx = gauss_legendre(n)
    z, wz = gauss_legendre(nz)
    pts, wts = [], []
    for w, ww in zip(z, wz):
        h = (1 - w)/2
        for v, wv in zip(x, wx):
            for u, wu in zip(x, wx):
                pts.append((u*h, v*h, w))
                wts.append(wu*wv*ww*h*h)
    return np.array(pts), np.array(wts)


def pyr_layers(rule, order):
    """The layered pyramid point sets of the reference's tables
    ``pyfr/quadrules/pyr/gauss-legendre-n*`` and
    ``gauss-legendre-lobatto-n*``: with n = order + 1, the k-th point of
    the n-point line rule (ascending) is the height z of a layer holding
    the (n - k)^2 tensor points of the (n - k)-point line rule scaled by
    (1 - z)/2 (x fastest, then y); layers in ascending z, except that the
    Lobatto set lists its apex, the one-point top layer, first."""
    n = order + 1
    zs, _ = RULES_1D[rule](n)
    layers = []
    for k, z in enumerate(zs):
        m = n - k
        if m == 1:
            xs = np.zeros(1)
        else:
            xs, _ = RULES_1D[rule](m)
        h = (1 - z)/2
        layers.append([(x*h, y*h, z) for y in xs for x in xs])
    if rule == 'gauss-legendre-lobatto' and n > 1:
        layers = [layers[-1]] + layers[:-1]
    return np.array([p for layer in layers for p in layer], dtype=float)


def quad_gauss(qdeg):
    return tensor_rule('gauss-legendre', qdeg//2 + 1, 2)


def hex_gauss(qdeg):
    return tensor_rule('gauss-legendre', qdeg//2 + 1, 3)


def line_gauss(qdeg):
    x, w = gauss_legendre(qdeg//2 + 1)
    return x[:, None], w


EXACT_RULES = {'line': line_gauss, 'tri': tri_gauss, 'quad': quad_gauss,
               'tet': tet_gauss, 'pri': pri_gauss, 'hex': hex_gauss,
               'pyr': pyr_gauss}


# ---------------------------------------------------------------------------
# Warp-and-blend nodes
# ---------------------------------------------------------------------------

# Optimised blending parameters of the tetrahedron, indexed by order
# (Warburton 2006, table 2; 1.0 beyond it).  The triangle uses the same
# values, so that the triangle nodes are exactly the face nodes of the
# tetrahedron and tet faces conform with triangular interfaces; this is
# also what the reference's triangle 'alpha-opt' points are.
_ALPHA = [0.0, 0.0, 0.0, 0.0, 0.1002, 1.1332, 1.5608, 1.3413, 1.2577,
          1.1603, 1.10153, 0.6080, 0.4523, 0.8856, 0.8717, 0.9655]


def _alpha(p):
    return _ALPHA[p] if p < len(_ALPHA) else 1.0


def _warp_factor(p, r):
    """Displacement along an edge that moves the p + 1 equispaced points
    onto the Gauss-Lobatto points, divided by the edge blend 1 - r^2
    (evaluated at the edge coordinate r in [-1, 1])."""
    gll, _ = gauss_legendre_lobatto(p + 1)
    req = np.linspace(-1, 1, p + 1)

    # Lagrange interpolant through the equispaced points of the shifts
    warp = np.zeros_like(r)
    for i in range(p + 1):
        li = np.ones_like(r)
        for j in range(p + 1):
            if j != i:
                li = li*(r - req[j])/(req[i] - req[j])
        warp += (gll[i] - req[i])*li

    inner = np.abs(r) < 1 - 1e-10
    return np.where(inner, warp/np.where(inner, 1 - r*r, 1.0), 0.0)


def _tri_shift(p, alpha, l1, l2, l3):
    """In-plane warp (dx, dy) of a point with barycentric coordinates
    (l1, l2, l3) of an equilateral triangle, summed over its three edges."""
    w1 = 4*l2*l3*_warp_factor(p, l3 - l2)*(1 + (alpha*l1)**2)
    w2 = 4*l1*l3*_warp_factor(p, l1 - l3)*(1 + (alpha*l2)**2)
    w3 = 4*l1*l2*_warp_factor(p, l2 - l1)*(1 + (alpha*l3)**2)
    c2, s2 = math.cos(2*math.pi/3), math.sin(2*math.pi/3)
    c4, s4 = math.cos(4*math.pi/3), math.sin(4*math.pi/3)
    return w1 + c2*w2 + c4*w3, s2*w2 + s4*w3


def _lattice(p, ndims):
    """Equispaced lattice of the order-p simplex, x fastest, as integer
    index tuples."""
    if ndims == 2:
        return [(i, j) for j in range(p + 1) for i in range(p + 1 - j)]
    return [(i, j, k) for k in range(p + 1) for j in range(p + 1 - k)
            for i in range(p + 1 - j - k)]


def alpha_opt_tri(p):
    """Warp-and-blend nodes of order p on the reference triangle."""
    if p == 0:
        return np.array([[-1/3, -1/3]])
    alpha = _alpha(p)
    ij = np.array(_lattice(p, 2), dtype=float)

    # Barycentric coordinates: l2 at (-1,-1), l3 at (1,-1), l1 at (-1,1)
    l3, l1 = ij[:, 0]/p, ij[:, 1]/p
    l2 = 1 - l1 - l3

    # Equilateral triangle with the same vertex correspondence
    x = -l2 + l3
    y = (-l2 - l3 + 2*l1)/math.sqrt(3)
    dx, dy = _tri_shift(p, alpha, l1, l2, l3)
    x, y = x + dx, y + dy

    # Back to the reference triangle
    b1 = (math.sqrt(3)*y + 1)/3
    b2 = (-3*x - math.sqrt(3)*y + 2)/6
    b3 = (3*x - math.sqrt(3)*y + 2)/6
    pts = np.stack([-b2 + b3 - b1, -b2 - b3 + b1], axis=1)
    return _snap(pts)


def alpha_opt_tet(p):
    """Warp-and-blend nodes of order p on the reference tetrahedron."""
    if p == 0:
        return np.array([[-0.5, -0.5, -0.5]])
    alpha = _alpha(p)
    ijk = np.array(_lattice(p, 3), dtype=float)
    r, s, t = (2*ijk/p - 1).T

    # Barycentric coordinates of the reference tetrahedron
    L1, L2 = (1 + t)/2, (1 + s)/2
    L3, L4 = -(1 + r + s + t)/2, (1 + r)/2

    # Regular tetrahedron with the matching vertices
    v1 = np.array([-1, -1/math.sqrt(3), -1/math.sqrt(6)])
    v2 = np.array([1, -1/math.sqrt(3), -1/math.sqrt(6)])
    v3 = np.array([0, 2/math.sqrt(3), -1/math.sqrt(6)])
    v4 = np.array([0, 0, 3/math.sqrt(6)])
    t1 = [v2 - v1, v2 - v1, v3 - v2, v3 - v1]
    t2 = [v3 - (v1 + v2)/2, v4 - (v1 + v2)/2, v4 - (v2 + v3)/2,
          v4 - (v1 + v3)/2]
    t1 = [a/np.linalg.norm(a) for a in t1]
    t2 = [a/np.linalg.norm(a) for a in t2]

    xyz = np.outer(L3, v1) + np.outer(L4, v2) + np.outer(L2, v3) + \
        np.outer(L1, v4)
    shift = np.zeros_like(xyz)
    tol = 1e-10
    faces = [(L1, L2, L3, L4), (L2, L1, L3, L4), (L3, L1, L4, L2),
             (L4, L1, L3, L2)]
    for f, (La, Lb, Lc, Ld) in enumerate(faces):
        # Warp within the face opposite to the vertex of La
        w1, w2 = _tri_shift(p, alpha, Lb, Lc, Ld)

        # Blend it into the volume
        blend = Lb*Lc*Ld
        denom = (Lb + La/2)*(Lc + La/2)*(Ld + La/2)
        big = denom > tol
        blend = np.where(big, (1 + (alpha*La)**2)*blend
                         / np.where(big, denom, 1.0), blend)
        shift += np.outer(blend*w1, t1[f]) + np.outer(blend*w2, t2[f])

        # Points on the face itself (but not on one of its edges) take the
        # face warp unblended
        onface = (La < tol) & ((Lb > tol).astype(int) + (Lc > tol)
                               + (Ld > tol) < 3)
        shift[onface] = (np.outer(w1[onface], t1[f])
                         + np.outer(w2[onface], t2[f]))

    xyz += shift

    # Back to the reference tetrahedron
    A = np.stack([(v2 - v1)/2, (v3 - v1)/2, (v4 - v1)/2], axis=1)
    rhs = xyz - (v2 + v3 + v4 - v1)/2
    pts = np.linalg.solve(A, rhs.T).T
    return _snap(pts)


def _snap(pts, tol=1e-14):
    """Give coordinates within ``tol`` of -1, 0 or 1 those exact values
    (vertex and edge points of the lattice land there analytically)."""
    out = pts.copy()
    for v in (-1.0, 0.0, 1.0):
        out[np.abs(out - v) < tol] = v
    return out


def parse_rule(text, ndims):
    """Points (and weights, if every point has one) of a rule written in
    the reference's tabulated text format."""
    t = re.sub(r'(?<=\))\s*,?\s*(?!$)', '\n', text)
    t = re.sub(r'\(|\)|,', ' ', t).strip()
    if t.startswith('[') and t.endswith(']'):
        t = t[1:-1]

    pts, wts = [], []
    for line in t.splitlines():
        vals = [float(v) for v in line.split()]
        if not vals:
            continue
        if len(vals) == ndims:
            pts.append(vals)
        elif len(vals) == ndims + 1:
            pts.append(vals[:-1])
            wts.append(vals[-1])
        else:
            raise ValueError('Invalid point in rule')
    if wts and len(wts) != len(pts):
        raise ValueError('Invalid number of weights')
    return np.array(pts, dtype=float), (np.array(wts) if wts else None)


_NDIMS = dict(line=1, tri=2, quad=2, tet=3, pri=3, hex=3, pyr=3)


def is_literal(rule):
    return not re.fullmatch(r'[a-zA-Z0-9\-~+]+', rule)


def point_set(kind, rule, order):
    """Nodal points of the order-``order`` polynomial space on ``kind``
    for the named (or literal) ``rule``."""
    n = order + 1
    if is_literal(rule):
        pts, _ = parse_rule(rule, _NDIMS[kind])
    elif kind in ('line', 'quad', 'hex') and rule in RULES_1D:
        pts, _ = tensor_rule(rule, n, _NDIMS[kind])
    elif kind == 'tri' and rule == 'alpha-opt':
        pts = alpha_opt_tri(order)
    elif kind == 'tet' and rule == 'alpha-opt':
        pts = alpha_opt_tet(order)
    elif kind == 'pyr' and rule in RULES_1D:
        pts = pyr_layers(rule, order)
    elif kind == 'pri' and '~' in rule:
        trule, lrule = rule.split('~')
        tp = point_set('tri', trule, order)
        lp, _ = RULES_1D[lrule](n)
        pts = np.array([[*q, z] for z in lp for q in tp])
    else:
        raise ValueError(f'No point set {rule!r} for {kind}')

    npts = {'line': n, 'quad': n**2, 'hex': n**3, 'tri': n*(n + 1)//2,
            'tet': n*(n + 1)*(n + 2)//6, 'pri': n*n*(n + 1)//2,
            'pyr': n*(n + 1)*(2*n + 1)//6}[kind]
    if len(pts) != npts:
        raise ValueError(f'Rule {rule!r} has {len(pts)} points; {kind} '
                         f'order {order} needs {npts}')
    return np.asarray(pts, dtype=float).reshape(npts, _NDIMS[kind])
