"""Orthonormal and nodal polynomial bases on the reference elements.

The flux-reconstruction operators are built from the same mathematical
objects as ``pyfr/polys.py`` (orthonormal Legendre products, Vandermonde
inversion to a nodal basis at the solution points,
``pyfr/polys.py:46-88`` and ``pyfr/polys.py:126-150,402-433``).  This
module is a fresh, vectorised statement of that mathematics: the nodal
basis that results is independent of how the modes are enumerated, so only
the ordering of the nodal points has to agree with the reference (x
fastest, then y, then z).

The pyramid's space (``pyfr/polys.py:333-402``) is not a set of Legendre
products; ``PyrBasis`` spans it with homogeneous Legendre polynomials and
orthonormalises them on the element, which reproduces the reference's
orthonormal pyramid modes.

The simplex and prism spaces (total degree <= p on the triangle and the
tetrahedron; total degree <= p in (x, y) times degree <= p in z on the
prism, the spaces of ``pyfr/polys.py:112-330``) are spanned here by
products of Legendre polynomials restricted to those degrees.  Unlike the
reference's collapsed-coordinate (Dubiner) modes these are not orthogonal
on the element, but they span the same space, have derivatives without
the collapsed coordinates' singular points, and are well conditioned at
the orders of interest; the nodal bases and operators are the same.  The
shapes that use them integrate with explicit mass matrices where the
reference relies on orthonormality.
"""

import itertools as it

import numpy as np


def legendre_orthonormal(order, x):
    """Values and first derivatives of the L2-orthonormal Legendre
    polynomials sqrt(k + 1/2) P_k(x) for k = 0..order.

    Returns two arrays of shape (order + 1, len(x)).
    """
    x = np.asarray(x, dtype=float)
    p = np.zeros((order + 1,) + x.shape)
    dp = np.zeros_like(p)

    p[0] = 1.0
    if order >= 1:
        p[1] = x
        dp[1] = 1.0

    # Bonnet recursion for P_k and the derivative identity
    # P'_k = k P_{k-1} + x P'_{k-1}
    for k in range(2, order + 1):
        p[k] = ((2*k - 1)*x*p[k - 1] - (k - 1)*p[k - 2]) / k
        dp[k] = k*p[k - 1] + x*dp[k - 1]

    scale = np.sqrt(np.arange(order + 1) + 0.5)
    shp = (-1,) + (1,)*x.ndim
    return scale.reshape(shp)*p, scale.reshape(shp)*dp


def space_modes(kind, order):
    """Multi-indices (Legendre degree per coordinate) spanning the
    polynomial space of order ``order`` on element type ``kind``."""
    p = order
    if kind == 'line':
        return [(i,) for i in range(p + 1)]
    if kind in ('quad', 'hex'):
        nd = 2 if kind == 'quad' else 3
        return [m[::-1] for m in it.product(range(p + 1), repeat=nd)]
    if kind == 'tri':
        return [(i, j) for j in range(p + 1) for i in range(p + 1 - j)]
    if kind == 'tet':
        return [(i, j, k) for k in range(p + 1) for j in range(p + 1 - k)
                for i in range(p + 1 - j - k)]
    if kind == 'pri':
        return [(i, j, k) for k in range(p + 1) for j in range(p + 1)
                for i in range(p + 1 - j)]
    raise ValueError(f'No polynomial space for {kind!r}')


class TensorProdBasis:
    """Basis of Legendre products of degree ``order`` in each of ``ndims``
    reference coordinates (orthonormal on the square/cube), or of the
    products listed in ``modes``, with a nodal basis at ``pts``."""

    def __init__(self, ndims, order, pts=None, modes=None):
        self.ndims = ndims
        self.order = order
        self.pts = None if pts is None else np.atleast_2d(pts)

        # Multi-indices of the modes
        if modes is None:
            modes = list(it.product(range(order + 1), repeat=ndims))
        self.modes = modes

    def _factors(self, pts):
        pts = np.atleast_2d(np.asarray(pts, dtype=float))
        if pts.shape[-1] != self.ndims:
            pts = pts.reshape(-1, self.ndims)

        return [legendre_orthonormal(self.order, pts[:, d])
                for d in range(self.ndims)]

    def ortho_basis_at(self, pts):
        """Orthonormal modes at ``pts``; shape (nmodes, npts)."""
        f = self._factors(pts)
        out = []
        for m in self.modes:
            v = f[0][0][m[0]].copy()
            for d in range(1, self.ndims):
                v *= f[d][0][m[d]]
            out.append(v)

        return np.array(out)

    def jac_ortho_basis_at(self, pts):
        """Reference-space gradients of the modes; shape
        (ndims, nmodes, npts)."""
        f = self._factors(pts)
        out = np.empty((self.ndims, len(self.modes), len(f[0][0][0])))
        for i, m in enumerate(self.modes):
            for g in range(self.ndims):
                v = np.ones_like(f[0][0][0])
                for d in range(self.ndims):
                    v = v*(f[d][1][m[d]] if d == g else f[d][0][m[d]])
                out[g, i] = v

        return out

    @property
    def vdm(self):
        return self.ortho_basis_at(self.pts)

    @property
    def invvdm(self):
        return np.linalg.inv(self.vdm)

    def nodal_basis_at(self, epts):
        """Lagrange basis of the nodal points evaluated at ``epts``;
        shape (nepts, nnodes)."""
        return (self.invvdm @ self.ortho_basis_at(epts)).T

    def jac_nodal_basis_at(self, epts):
        """Gradient of the Lagrange basis at ``epts``; shape
        (ndims, nnodes, nepts)."""
        return self.invvdm @ self.jac_ortho_basis_at(epts)


def homogeneous_legendre(order, x, s):
    """H_k(x, s) = s^k P_k(x/s), k = 0..order, with the partial derivatives
    dH_k/dx and dH_k/ds: Bonnet's recursion multiplied through by s^k,
    H_k = ((2k - 1) x H_(k-1) - (k - 1) s^2 H_(k-2))/k, which keeps every
    H_k a polynomial in x and s (no division by s, so the pyramid's apex
    s = 0 is an ordinary point).  Three arrays of shape
    (order + 1, len(x))."""
    x, s = np.broadcast_arrays(np.asarray(x, dtype=float),
                               np.asarray(s, dtype=float))
    h = np.zeros((order + 1,) + x.shape)
    hx, hs = np.zeros_like(h), np.zeros_like(h)
    h[0] = 1.0
    if order >= 1:
        h[1], hx[1] = x, 1.0
    for k in range(2, order + 1):
        a, b = 2*k - 1, k - 1
        h[k] = (a*x*h[k - 1] - b*s*s*h[k - 2])/k
        hx[k] = (a*(h[k - 1] + x*hx[k - 1]) - b*s*s*hx[k - 2])/k
        hs[k] = (a*x*hs[k - 1] - b*(2*s*h[k - 2] + s*s*hs[k - 2]))/k
    return h, hx, hs


class PyrBasis(TensorProdBasis):
    """The pyramid's polynomial space of order p (``pyfr/polys.py:333-402``):
    spanned by (1 - z)^(i+j) P_i(2x/(1 - z)) P_j(2y/(1 - z)) times every
    polynomial in z of degree <= p - max(i, j), for 0 <= i, j <= p.  With
    s = (1 - z)/2 the first factor is 2^(i+j) H_i(x, s) H_j(y, s) for the
    homogeneous Legendre polynomials H, so the modes here are
    H_i(x, s) H_j(y, s) L_k(z) with L_k the orthonormal Legendre
    polynomials, k <= p - max(i, j): polynomials (the reference's
    collapsed-coordinate modes, orthonormal on the pyramid, span the same
    space; the nodal basis at the solution points is the same).  They are
    made orthonormal on the pyramid by a Gram-Schmidt step (the Cholesky
    factor of their Gram matrix, integrated exactly), which keeps the
    Vandermonde matrices as well conditioned as the reference's.  The mode
    tuples (i, j, k) are listed in the reference's order."""

    def __init__(self, order, pts=None):
        from pyfr_gb300.quadrules import pyr_gauss
        modes = [(i, j, k) for i in range(order + 1)
                 for j in range(order + 1)
                 for k in range(order - max(i, j) + 1)]
        super().__init__(3, order, pts, modes)
        self._orth = np.eye(len(modes))
        qp, qw = pyr_gauss(4*order)
        for _ in range(2):          # twice: Gram-Schmidt's reorthogonalisation
            raw = self.ortho_basis_at(qp)
            c = np.linalg.cholesky((raw*qw) @ raw.T)
            self._orth = np.linalg.solve(c, self._orth)

    def _parts(self, pts):
        pts = np.atleast_2d(np.asarray(pts, dtype=float)).reshape(-1, 3)
        x, y, z = pts.T
        s = (1 - z)/2
        return (homogeneous_legendre(self.order, x, s),
                homogeneous_legendre(self.order, y, s),
                legendre_orthonormal(self.order, z))

    def ortho_basis_at(self, pts):
        (hx, _, _), (hy, _, _), (lz, _) = self._parts(pts)
        return self._orth @ np.array([hx[i]*hy[j]*lz[k]
                                      for i, j, k in self.modes])

    def jac_ortho_basis_at(self, pts):
        (hx, hxx, hxs), (hy, hyy, hys), (lz, dlz) = self._parts(pts)
        out = np.empty((3, len(self.modes), hx.shape[1]))
        for m, (i, j, k) in enumerate(self.modes):
            out[0, m] = hxx[i]*hy[j]*lz[k]
            out[1, m] = hx[i]*hyy[j]*lz[k]
            # d/dz = -1/2 d/ds on the H factors
            out[2, m] = (hx[i]*hy[j]*dlz[k] -
                         0.5*(hxs[i]*hy[j] + hx[i]*hys[j])*lz[k])
        return self._orth @ out


def tidy(arr, tol=1e-10):
    """Flush entries below ``tol`` to exact zero and give entries whose
    magnitudes agree to a relative ``tol`` one common magnitude.

    Operator matrices in the reference go through the same kind of clean-up
    (``pyfr/nputil.py:23-60``), so that analytically-zero entries are exact
    zeros (the sparsity pattern the operator kernels exploit) and entries
    equal by symmetry are bit-identical.
    """
    a = np.array(arr, dtype=float, copy=True)
    a[np.abs(a) < tol] = 0.0

    flat = a.reshape(-1)
    mag = np.abs(flat)
    order = np.argsort(mag, kind='stable')
    smag = mag[order]

    # Split the sorted magnitudes into runs of near-equal values
    brk = ~np.isclose(smag[1:], smag[:-1], rtol=tol, atol=0.1*tol)
    starts = np.concatenate([[0], np.flatnonzero(brk) + 1])
    ends = np.concatenate([starts[1:], [len(smag)]])
    for s, e in zip(starts, ends):
        if e - s > 1:
            rep = np.median(smag[s:e])
            idx = order[s:e]
            flat[idx] = np.copysign(rep, flat[idx])

    return a


def jacobi_orthonormal(order, a, b, x):
    """Jacobi polynomials P_k^(a,b)(x), k = 0..order, normalised to unit
    norm under the weight (1 - x)^a (1 + x)^b on [-1, 1]; shape
    (order + 1, len(x)).  The standard three-term recurrence in its
    orthonormal form (as in Hesthaven and Warburton, Nodal Discontinuous
    Galerkin Methods, 2008, appendix A)."""
    from math import gamma as G
    x = np.asarray(x, dtype=float)
    p = np.zeros((order + 1,) + x.shape)
    g0 = 2**(a + b + 1)/(a + b + 1)*G(a + 1)*G(b + 1)/G(a + b + 1)
    p[0] = 1/np.sqrt(g0)
    if order == 0:
        return p
    g1 = (a + 1)*(b + 1)/(a + b + 3)*g0
    p[1] = ((a + b + 2)*x/2 + (a - b)/2)/np.sqrt(g1)
    aold = 2/(2 + a + b)*np.sqrt((a + 1)*(b + 1)/(a + b + 3))
    for n in range(1, order):
        h1 = 2*n + a + b
        anew = 2/(h1 + 2)*np.sqrt((n + 1)*(n + 1 + a + b)*(n + 1 + a) *
                                  (n + 1 + b)/((h1 + 1)*(h1 + 3)))
        bnew = -(a*a - b*b)/(h1*(h1 + 2))
        p[n + 1] = ((x - bnew)*p[n] - aold*p[n - 1])/anew
        aold = anew
    return p


class SimplexOrthoBasis:
    """The collapsed-coordinate orthonormal (Proriol-Koornwinder-Dubiner)
    bases of the triangle, tetrahedron and prism, with their degree tuples
    in the reference's order (``pyfr/polys.py:112-330``): on the triangle
    psi_ij = sqrt(2) P_i(a) P_j^(2i+1,0)(b) (1 - b)^i, on the tetrahedron
    psi_ijk = 2 sqrt(2) P_i(a) P_j^(2i+1,0)(b) (1 - b)^i
    P_k^(2i+2j+2,0)(c) (1 - c)^(i+j), on the prism the triangle's modes
    times the line's, each factor orthonormal (Sherwin and Karniadakis,
    Spectral/hp Element Methods, 2005, ch. 3; Hesthaven and Warburton
    2008, ch. 6 and 10).  Orthonormal on the reference elements; used where
    a filter or sensor groups modes by degree, which depends on the basis
    (the operators do not)."""

    def __init__(self, kind, order, pts=None):
        self.kind, self.order = kind, order
        p = order
        if kind == 'tri':
            self.degrees = [(i, j) for i in range(p + 1)
                            for j in range(p - i + 1)]
        elif kind == 'tet':
            self.degrees = [(i, j, k) for i in range(p + 1)
                            for j in range(p - i + 1)
                            for k in range(p - i - j + 1)]
        elif kind == 'pri':
            self.degrees = [(i, j, k) for i in range(p + 1)
                            for j in range(p - i + 1) for k in range(p + 1)]
        else:
            raise ValueError(f'No simplex basis for {kind!r}')
        self.pts = None if pts is None else np.asarray(pts, dtype=float)

    @staticmethod
    def _tri(p, r, s):
        with np.errstate(divide='ignore', invalid='ignore'):
            a = np.where(s != 1, 2*(1 + r)/(1 - s) - 1, -1.0)
        pa = jacobi_orthonormal(p, 0, 0, a)
        out = []
        for i in range(p + 1):
            pb = jacobi_orthonormal(p - i, 2*i + 1, 0, s)
            for j in range(p - i + 1):
                out.append(np.sqrt(2)*pa[i]*pb[j]*(1 - s)**i)
        return out

    def ortho_basis_at(self, pts):
        pts = np.atleast_2d(np.asarray(pts, dtype=float))
        p = self.order
        if self.kind == 'tri':
            r, s = pts.T
            return np.array(self._tri(p, r, s))
        if self.kind == 'pri':
            r, s, t = pts.T
            tri = self._tri(p, r, s)
            line = jacobi_orthonormal(p, 0, 0, t)
            return np.array([f*line[k] for f in tri for k in range(p + 1)])
        r, s, t = pts.T
        with np.errstate(divide='ignore', invalid='ignore'):
            a = np.where(s + t != 0, -2*(1 + r)/(s + t) - 1, -1.0)
            b = np.where(t != 1, 2*(1 + s)/(1 - t) - 1, -1.0)
        pa = jacobi_orthonormal(p, 0, 0, a)
        out = []
        for i in range(p + 1):
            pb = jacobi_orthonormal(p - i, 2*i + 1, 0, b)
            for j in range(p - i + 1):
                pc = jacobi_orthonormal(p - i - j, 2*(i + j + 1), 0, t)
                for k in range(p - i - j + 1):
                    out.append(2*np.sqrt(2)*pa[i]*pb[j]*(1 - b)**i *
                               pc[k]*(1 - t)**(i + j))
        return np.array(out)

    @property
    def vdm(self):
        return self.ortho_basis_at(self.pts)

    @property
    def modes(self):
        return self.degrees


def modal_basis(shape):
    """The orthonormal modal basis whose degree groups a filter or sensor
    works with: the Legendre products of a quadrilateral or hexahedron and
    the pyramid's orthonormalised modes (the shapes' own bases), the
    collapsed-coordinate bases of the other types.
    Returns (basis at the solution points, degree tuples of its modes,
    degree tuples of the basis one order lower)."""
    if shape.name in ('quad', 'hex'):
        ub = shape.ubasis
        lower = [m for m in ub.modes if max(m) < shape.order]
        return ub, list(ub.modes), lower
    if shape.name == 'pyr':
        # Orthonormalised in the reference's mode order, the pyramid's
        # basis is the reference's orthonormal one
        lower = PyrBasis(shape.order - 1).modes if shape.order > 0 else []
        return shape.ubasis, list(shape.ubasis.modes), lower
    b = SimplexOrthoBasis(shape.name, shape.order, shape.upts)
    lower = SimplexOrthoBasis(shape.name, shape.order - 1).degrees \
        if shape.order > 0 else []
    return b, b.degrees, lower

