"""Reference elements and flux-reconstruction operator matrices.

Each shape supplies the solution points (``upts``), the flux points on its
faces (``fpts``) with their outward reference normals, and the operator
matrices that the right-hand side applies:

* ``M0`` (nfpts x nupts): interpolate the solution to the flux points;
* ``M1`` (nupts x ndims*nupts): reference-space divergence of a vector
  field held at the solution points;
* ``M2`` (nfpts x ndims*nupts): normal component of that field at the flux
  points;
* ``M3`` (nupts x nfpts): the correction (lifting) operator, here the DG
  correction obtained by L2-projecting the face nodal basis onto the
  element's orthonormal basis;
* ``M4`` (ndims*nupts x nupts): reference gradient of a scalar field;
* ``M6`` (ndims*nupts x nfpts): normal-weighted lift.

These follow the definitions of ``pyfr/shapes.py:80-125`` and
``pyfr/shapes.py:232-259`` (the lifting coefficients), with the same point
orderings, face orderings and normals (``pyfr/shapes.py:341-438``) so that
operators, element data and interface maps line up one-to-one with the
reference.  Only tensor-product shapes (quad, hex) with Gauss-Legendre or
Gauss-Legendre-Lobatto points are provided.
"""

from functools import cached_property
import itertools as it
import re

import numpy as np

from pyfr_gb300.polys import TensorProdBasis, tidy


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


_RULES_1D = {
    'gauss-legendre': gauss_legendre,
    'gauss-legendre-lobatto': gauss_legendre_lobatto,
}


def tensor_rule(name, n1d, ndims):
    """Tensor-product rule with the first coordinate varying fastest, the
    ordering of the tabulated rules in ``pyfr/quadrules/{quad,hex}``."""
    x, w = _RULES_1D[name](n1d)
    pts = np.array([p[::-1] for p in it.product(x, repeat=ndims)])
    wts = np.array([np.prod(q) for q in it.product(w, repeat=ndims)])
    return pts.reshape(-1, ndims), wts


def _proj(fn, pts):
    pts = np.atleast_2d(np.asarray(pts, dtype=float).T)
    cols = np.broadcast_arrays(*fn(*pts))
    return np.vstack(cols).T.astype(float)


class TensorProdShape:
    name = None
    ndims = None
    faces = None
    facekind = None

    def __init__(self, order, upts_rule='gauss-legendre',
                 fpts_rule='gauss-legendre'):
        self.order = order
        self.upts_rule = upts_rule
        self.fpts_rule = fpts_rule

        self.upts, _ = tensor_rule(upts_rule, order + 1, self.ndims)
        self.ubasis = TensorProdBasis(self.ndims, order, self.upts)

    # Vertex (linear shape point) ordering: x fastest; std_ele(1)
    @cached_property
    def linspts(self):
        return np.array([p[::-1] for p in it.product([-1.0, 1.0],
                                                      repeat=self.ndims)])

    @property
    def nupts(self):
        return (self.order + 1)**self.ndims

    @cached_property
    def nfacefpts(self):
        return [(self.order + 1)**(self.ndims - 1)]*len(self.faces)

    @property
    def nfpts(self):
        return sum(self.nfacefpts)

    @cached_property
    def facefpts(self):
        off = np.cumsum([0] + self.nfacefpts)
        return [list(range(off[i], off[i + 1]))
                for i in range(len(self.faces))]

    @cached_property
    def _face_rule(self):
        return tensor_rule(self.fpts_rule, self.order + 1, self.ndims - 1)

    @cached_property
    def fpts(self):
        fp, _ = self._face_rule
        return np.vstack([_proj(proj, fp) for proj, norm in self.faces])

    @cached_property
    def fpts_wts(self):
        _, fw = self._face_rule
        return np.hstack([fw]*len(self.faces))

    @cached_property
    def norm_fpts(self):
        return np.vstack([[norm]*n for (proj, norm), n
                          in zip(self.faces, self.nfacefpts)]).astype(float)

    @cached_property
    def facebasis(self):
        fp, _ = self._face_rule
        return TensorProdBasis(self.ndims - 1, self.order, fp)

    @cached_property
    def lift_coeffs(self):
        """Modal coefficients (nfpts x nmodes) of the DG lifting functions:
        the face nodal basis integrated against the element's orthonormal
        modes restricted to the face (exact Gauss-Legendre quadrature)."""
        qp, qw = tensor_rule('gauss-legendre', self.order + 1, self.ndims - 1)
        lq = self.facebasis.nodal_basis_at(qp)          # (nq, nfacefpts)

        blocks = []
        for proj, norm in self.faces:
            mq = self.ubasis.ortho_basis_at(_proj(proj, qp))   # (nmodes, nq)
            blocks.append((lq*qw[:, None]).T @ mq.T)
        return np.vstack(blocks)

    # Operator matrices -----------------------------------------------------

    @cached_property
    def m0(self):
        return tidy(self.ubasis.nodal_basis_at(self.fpts))

    @cached_property
    def m1(self):
        jac = self.ubasis.jac_nodal_basis_at(self.upts)    # (d, nupts_j, e)
        return tidy(np.moveaxis(jac, 2, 0).reshape(self.nupts, -1))

    @cached_property
    def m2(self):
        m = self.norm_fpts[:, :, None]*self.m0[:, None, :]
        return tidy(m.reshape(self.nfpts, -1))

    @cached_property
    def m3(self):
        return tidy((self.lift_coeffs @ self.ubasis.ortho_basis_at(self.upts)).T)

    @cached_property
    def m4(self):
        m = self.m1.reshape(self.nupts, self.ndims, self.nupts)
        return tidy(m.swapaxes(0, 1).reshape(-1, self.nupts))

    @cached_property
    def m6(self):
        m = self.norm_fpts.T[:, None, :]*self.m3[None, :, :]
        return tidy(m.reshape(-1, self.nfpts))

    def opmat(self, expr):
        """Evaluate an operator expression such as ``'M1 - M3*M2'``."""
        e = expr.lower().replace('*', '@')
        if not re.fullmatch(r'[m0-9\-+@() ]+', e):
            raise ValueError(f'Invalid operator matrix expression {expr!r}')

        names = {m: getattr(self, m) for m in set(re.findall(r'm\d+', e))}
        return tidy(eval(e, {'__builtins__': {}}, names))

    # Geometry of linear (affine or multilinear) elements --------------------

    def shape_fn(self, x):
        """Multilinear shape functions of the vertices at points ``x``;
        shape (npts, nverts)."""
        x = np.atleast_2d(x)
        v = self.linspts
        return np.prod(1 + x[:, None, :]*v[None, :, :], axis=2) / 2**self.ndims

    def shape_jac(self, x):
        """d(shape fn)/d(xi_i); shape (npts, ndims, nverts)."""
        x = np.atleast_2d(x)
        v = self.linspts
        out = np.empty((len(x), self.ndims, len(v)))
        for i in range(self.ndims):
            t = np.ones((len(x), len(v)))
            for d in range(self.ndims):
                t = t*(v[None, :, d] if d == i else 1 + x[:, None, d]*v[None, :, d])
            out[:, i] = t / 2**self.ndims
        return out


class QuadShape(TensorProdShape):
    name = 'quad'
    ndims = 2
    facekind = 'line'

    # (reference-to-face projection, outward normal) in reference order
    faces = [
        (lambda s: (s, -1), (0, -1)),
        (lambda s: (1, s), (1, 0)),
        (lambda s: (s, 1), (0, 1)),
        (lambda s: (-1, s), (-1, 0)),
    ]


class HexShape(TensorProdShape):
    name = 'hex'
    ndims = 3
    facekind = 'quad'

    faces = [
        (lambda s, t: (s, t, -1), (0, 0, -1)),
        (lambda s, t: (s, -1, t), (0, -1, 0)),
        (lambda s, t: (1, s, t), (1, 0, 0)),
        (lambda s, t: (s, 1, t), (0, 1, 0)),
        (lambda s, t: (-1, s, t), (-1, 0, 0)),
        (lambda s, t: (s, t, 1), (0, 0, 1)),
    ]


SHAPES = {'quad': QuadShape, 'hex': HexShape}


def get_shape(name, order, upts_rule='gauss-legendre',
              fpts_rule='gauss-legendre'):
    try:
        return SHAPES[name](order, upts_rule, fpts_rule)
    except KeyError:
        raise ValueError(f'Unsupported element type {name!r}') from None


def adjugate_det(J):
    """Adjugate (transposed cofactor) metric S and determinant of Jacobians
    J[p, i, j, e] = dx_j/dxi_i: S[p, i, k] is the cross product of rows
    i+1 and i+2 (3-D) so that S^T J = |J| I, the metric terms of
    pyfr/solvers/baseadvec/kernels/smats.mako:3-25."""
    S = np.empty_like(J)
    if J.shape[1] == 2:
        S[:, 0, 0], S[:, 0, 1] = J[:, 1, 1], -J[:, 1, 0]
        S[:, 1, 0], S[:, 1, 1] = -J[:, 0, 1], J[:, 0, 0]
        d = S[:, 0, 0]*S[:, 1, 1] - S[:, 0, 1]*S[:, 1, 0]
    else:
        Jc = [[np.ascontiguousarray(J[:, i, j]) for j in range(3)]
              for i in range(3)]
        for i in range(3):
            a, b = Jc[(i + 1) % 3], Jc[(i + 2) % 3]
            for k in range(3):
                k1, k2 = (k + 1) % 3, (k + 2) % 3
                S[:, i, k] = a[k1]*b[k2] - a[k2]*b[k1]
        d = Jc[0][0]*S[:, 0, 0] + Jc[0][1]*S[:, 0, 1] + Jc[0][2]*S[:, 0, 2]
    return S, d
