"""Reference elements and flux-reconstruction operator matrices.

Each shape supplies the solution points (``upts``), the flux points on its
faces (``fpts``) with their outward reference normals, and the operator
matrices that the right-hand side applies:

* ``M0`` (nfpts x nupts): interpolate the solution to the flux points;
* ``M1`` (nupts x ndims*nupts): reference-space divergence of a vector
  field held at the solution points;
* ``M2`` (nfpts x ndims*nupts): normal component of that field at the flux
  points;
* ``M3`` (nupts x nfpts): the correction (lifting) operator, the DG
  correction: the lift g_f of flux point f is the polynomial of the
  solution space with  int_E g_f phi = int_face L_f phi  for every phi of
  the space (L_f the face's nodal basis function of f);
* ``M4`` (ndims*nupts x nupts): reference gradient of a scalar field;
* ``M6`` (ndims*nupts x nfpts): normal-weighted lift.

These follow the definitions of ``pyfr/shapes.py:80-125`` and
``pyfr/shapes.py:232-259`` (the lifting coefficients), with the same face
orderings, face parametrisations and normals (``pyfr/shapes.py:341-566``)
so that operators, element data and interface maps line up one-to-one with
the reference.  Quadrilaterals and hexahedra (Gauss-Legendre or
Gauss-Legendre-Lobatto points), triangles, tetrahedra ('alpha-opt' points),
prisms (triangle points times line points) and pyramids (layered
Gauss-Legendre or Gauss-Legendre-Lobatto points) are provided; any shape
also takes literal point sets in the reference's rule text format.

The tensor-product shapes form the lift from orthonormal modes, as the
reference does; the simplex and prism shapes solve with the element mass
matrix instead (same lift, basis-independent), both with quadrature exact
for the integrands.
"""

from functools import cached_property
import re

import numpy as np

from pyfr_gb300.polys import PyrBasis, TensorProdBasis, space_modes, tidy
from pyfr_gb300.quadrules import (EXACT_RULES, gauss_legendre,
                                  gauss_legendre_lobatto, point_set,
                                  tensor_rule)

__all__ = ['gauss_legendre', 'gauss_legendre_lobatto', 'tensor_rule',
           'get_shape', 'adjugate_det', 'linear_shape_jac', 'SHAPES']


def _proj(fn, pts):
    pts = np.atleast_2d(np.asarray(pts, dtype=float).T)
    cols = np.broadcast_arrays(*fn(*pts))
    return np.vstack(cols).T.astype(float)


FACE_KIND = {'quad': 'line', 'hex': 'quad', 'tri': 'line', 'tet': 'tri'}


class BaseShape:
    name = None
    ndims = None

    # (face kind, reference-to-face projection, outward normal), in the
    # reference's face order
    faces = None

    # Largest total degree of the solution space, in multiples of the
    # order (the pyramid's modes reach twice the order); it sets the
    # degrees of the quadratures that integrate mass matrices and lifts
    space_degree = 1

    def __init__(self, order, upts_rule='gauss-legendre',
                 fpts_rule='gauss-legendre'):
        self.order = order
        self.upts_rule = upts_rule
        kinds = {k for k, _, _ in self.faces}
        if isinstance(fpts_rule, str):
            fpts_rule = {k: fpts_rule for k in kinds}
        self.fpts_rules = {k: fpts_rule[k] for k in kinds}

        self.upts = point_set(self.name, upts_rule, order)
        self.ubasis = self._solution_basis()

    def _solution_basis(self):
        return TensorProdBasis(self.ndims, self.order, self.upts,
                               self._modes(self.name))

    def _modes(self, kind):
        return space_modes(kind, self.order)

    @property
    def fpts_rule(self):
        (r,) = set(self.fpts_rules.values())
        return r

    @property
    def nupts(self):
        return len(self.upts)

    @property
    def facekind(self):
        (k,) = {k for k, _, _ in self.faces}
        return k

    @cached_property
    def std_face_pts(self):
        """The face points of the flux-point rules in face coordinates
        (the points of the face bases)."""
        return {k: point_set(k, r, self.order)
                for k, r in self.fpts_rules.items()}

    @cached_property
    def face_pts(self):
        """Flux points of each face kind in face coordinates: those of
        the flux-point rule, or with surface-flux anti-aliasing the points
        of the face quadrature rule."""
        if getattr(self, '_surf_rules', None):
            return {k: pw[0] for k, pw in self._surf_rules.items()}
        return self.std_face_pts

    def set_surf_rules(self, rules):
        """Surface-flux anti-aliasing (pyfr/shapes.py:103-113,194-227):
        the flux points become the points of a quadrature rule per face
        kind, rules = {kind: (pts, wts)}, and the correction lift takes the
        L2 projection of the face flux onto the face basis."""
        self._surf_rules = {k: (np.asarray(p, dtype=float).reshape(
            len(w), -1), np.asarray(w, dtype=float))
            for k, (p, w) in rules.items()}
        for k in ('face_pts', 'nfacefpts', 'facefpts', 'fpts', 'norm_fpts',
                  'm0', 'm2', 'm3', 'm6', 'fpts_wts'):
            self.__dict__.pop(k, None)

    @cached_property
    def nfacefpts(self):
        return [len(self.face_pts[k]) for k, _, _ in self.faces]

    @property
    def nfpts(self):
        return sum(self.nfacefpts)

    @cached_property
    def facefpts(self):
        off = np.cumsum([0] + self.nfacefpts)
        return [list(range(off[i], off[i + 1]))
                for i in range(len(self.faces))]

    @cached_property
    def fpts(self):
        return np.vstack([_proj(proj, self.face_pts[k])
                          for k, proj, norm in self.faces])

    @cached_property
    def norm_fpts(self):
        return np.vstack([[norm]*n for (k, proj, norm), n
                          in zip(self.faces, self.nfacefpts)]).astype(float)

    @cached_property
    def facebases(self):
        return {k: TensorProdBasis(self.ndims - 1, self.order, p,
                                   self._modes(k))
                for k, p in self.std_face_pts.items()}

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
        m = self._lift_at_upts()
        if getattr(self, '_surf_rules', None):
            # proj_l2 of each face: the face basis' nodal values of the L2
            # projection of values at the face quadrature points (the face
            # bases are orthonormal Legendre products)
            from scipy.linalg import block_diag
            blocks = []
            for kind, _, _ in self.faces:
                fb = self.facebases[kind]
                qp, qw = self._surf_rules[kind]
                blocks.append(fb.vdm.T @ (qw[None, :]*fb.ortho_basis_at(qp)))
            m = m @ block_diag(*blocks)
        return tidy(m)

    @cached_property
    def m4(self):
        m = self.m1.reshape(self.nupts, self.ndims, self.nupts)
        return tidy(m.swapaxes(0, 1).reshape(-1, self.nupts))

    @cached_property
    def m6(self):
        m = self.norm_fpts.T[:, None, :]*self.m3[None, :, :]
        return tidy(m.reshape(-1, self.nfpts))

    # Flux anti-aliasing (pyfr/shapes.py:126-138) ------------------------

    def set_qrule(self, pts, wts):
        """Quadrature rule of the element for flux anti-aliasing."""
        self._qrule = (np.asarray(pts, dtype=float).reshape(-1, self.ndims),
                       np.asarray(wts, dtype=float))
        for k in ('m7', 'm8'):
            self.__dict__.pop(k, None)

    @property
    def qrule(self):
        if getattr(self, '_qrule', None) is None:
            if not isinstance(self, TensorProdShape):
                raise ValueError(f'{self.name}: anti-aliasing needs a '
                                 'quadrature rule (quad-pts)')
            # The reference's default: Gauss-Legendre, (p + 2)^ndims points
            self._qrule = tensor_rule('gauss-legendre', self.order + 2,
                                      self.ndims)
        return self._qrule

    @property
    def qpts(self):
        return self.qrule[0]

    @property
    def nqpts(self):
        return len(self.qpts)

    @cached_property
    def m7(self):
        """Interpolation from the solution points to the quadrature
        points."""
        return tidy(self.ubasis.nodal_basis_at(self.qpts))

    @cached_property
    def m8(self):
        """L2 projection of values at the quadrature points onto the
        solution space, at the solution points: with the element's exact
        mass matrix M, c = M^-1 sum_q w_q l_i(x_q) f_q (the reference's
        orthonormal-mode form, pyfr/shapes.py:17-19,131-133)."""
        qp, qw = EXACT_RULES[self.name](2*self.space_degree*self.order)
        L = self.ubasis.nodal_basis_at(qp)
        mass = L.T @ (qw[:, None]*L)
        lq = self.ubasis.nodal_basis_at(self.qpts)          # (nq, nupts)
        pts, wts = self.qrule
        return tidy(np.linalg.solve(mass, lq.T*wts[None, :]))

    @property
    def m9(self):
        m8 = self.m8
        nu, nq = m8.shape
        out = np.zeros((self.ndims*nu, self.ndims*nq))
        for d in range(self.ndims):
            out[d*nu:(d + 1)*nu, d*nq:(d + 1)*nq] = m8
        return out

    def opmat(self, expr):
        """Evaluate an operator expression such as ``'M1 - M3*M2'``."""
        e = expr.lower().replace('*', '@')
        if not re.fullmatch(r'[m0-9\-+@() ]+', e):
            raise ValueError(f'Invalid operator matrix expression {expr!r}')

        names = {m: getattr(self, m) for m in set(re.findall(r'm\d+', e))}
        return tidy(eval(e, {'__builtins__': {}}, names))

    def _lift_at_upts(self):
        """Lift via the element mass matrix of the nodal basis:
        M c_f = b_f with M_ij = int_E l_i l_j, b_f,i = int_face L_f l_i
        (face integrals in the face parametrisation, whose measure the
        unnormalised reference normals account for); returns the
        (nupts, nfpts) values g_f(upts) = c_f."""
        f = self.space_degree
        qp, qw = EXACT_RULES[self.name](2*f*self.order)
        L = self.ubasis.nodal_basis_at(qp)                 # (nq, nupts)
        mass = L.T @ (qw[:, None]*L)

        cols = []
        for kind, proj, norm in self.faces:
            fq, fw = EXACT_RULES[kind]((f + 1)*self.order)
            lf = self.facebases[kind].nodal_basis_at(fq)   # (nfq, nff)
            le = self.ubasis.nodal_basis_at(_proj(proj, fq))
            cols.append(le.T @ (fw[:, None]*lf))
        return np.linalg.solve(mass, np.hstack(cols))

    # Geometry of linear elements --------------------------------------------

    def shape_fn(self, x):
        """Linear shape functions of the vertices at points ``x``;
        shape (npts, nverts)."""
        return linear_shape_fn(self.name, np.atleast_2d(x))

    def shape_jac(self, x):
        """d(shape fn)/d(xi_i); shape (npts, ndims, nverts)."""
        return linear_shape_jac(self.name, np.atleast_2d(x))


class TensorProdShape(BaseShape):
    # Vertex (linear shape point) ordering: x fastest; std_ele(1)
    @cached_property
    def linspts(self):
        return np.array(VERTICES[self.name], dtype=float)

    @cached_property
    def _face_rule(self):
        return tensor_rule(self.fpts_rule, self.order + 1, self.ndims - 1)

    @cached_property
    def fpts_wts(self):
        if getattr(self, '_surf_rules', None):
            return np.hstack([self._surf_rules[k][1] for k, _, _ in self.faces])
        _, fw = self._face_rule
        return np.hstack([fw]*len(self.faces))

    @cached_property
    def facebasis(self):
        return self.facebases[self.facekind]

    @cached_property
    def lift_coeffs(self):
        """Modal coefficients (nfpts x nmodes) of the DG lifting functions:
        the face nodal basis integrated against the element's orthonormal
        modes restricted to the face (exact Gauss-Legendre quadrature)."""
        qp, qw = tensor_rule('gauss-legendre', self.order + 1, self.ndims - 1)
        lq = self.facebasis.nodal_basis_at(qp)          # (nq, nfacefpts)

        blocks = []
        for kind, proj, norm in self.faces:
            mq = self.ubasis.ortho_basis_at(_proj(proj, qp))   # (nmodes, nq)
            blocks.append((lq*qw[:, None]).T @ mq.T)
        return np.vstack(blocks)

    def _lift_at_upts(self):
        return (self.lift_coeffs @ self.ubasis.ortho_basis_at(self.upts)).T

    def _modes(self, kind):
        return None


class SimplexLikeShape(BaseShape):
    @cached_property
    def linspts(self):
        return np.array(VERTICES[self.name], dtype=float)


class QuadShape(TensorProdShape):
    name = 'quad'
    ndims = 2

    faces = [
        ('line', lambda s: (s, -1), (0, -1)),
        ('line', lambda s: (1, s), (1, 0)),
        ('line', lambda s: (s, 1), (0, 1)),
        ('line', lambda s: (-1, s), (-1, 0)),
    ]


class HexShape(TensorProdShape):
    name = 'hex'
    ndims = 3

    faces = [
        ('quad', lambda s, t: (s, t, -1), (0, 0, -1)),
        ('quad', lambda s, t: (s, -1, t), (0, -1, 0)),
        ('quad', lambda s, t: (1, s, t), (1, 0, 0)),
        ('quad', lambda s, t: (s, 1, t), (0, 1, 0)),
        ('quad', lambda s, t: (-1, s, t), (-1, 0, 0)),
        ('quad', lambda s, t: (s, t, 1), (0, 0, 1)),
    ]


class TriShape(SimplexLikeShape):
    name = 'tri'
    ndims = 2

    faces = [
        ('line', lambda s: (s, -1), (0, -1)),
        ('line', lambda s: (-s, s), (1, 1)),
        ('line', lambda s: (-1, s), (-1, 0)),
    ]


class TetShape(SimplexLikeShape):
    name = 'tet'
    ndims = 3

    faces = [
        ('tri', lambda s, t: (s, t, -1), (0, 0, -1)),
        ('tri', lambda s, t: (s, -1, t), (0, -1, 0)),
        ('tri', lambda s, t: (-1, t, s), (-1, 0, 0)),
        ('tri', lambda s, t: (s, t, -s - t - 1), (1, 1, 1)),
    ]


class PriShape(SimplexLikeShape):
    name = 'pri'
    ndims = 3

    faces = [
        ('tri', lambda s, t: (s, t, -1), (0, 0, -1)),
        ('tri', lambda s, t: (s, t, 1), (0, 0, 1)),
        ('quad', lambda s, t: (s, -1, t), (0, -1, 0)),
        ('quad', lambda s, t: (-s, s, t), (1, 1, 0)),
        ('quad', lambda s, t: (-1, s, t), (-1, 0, 0)),
    ]


class PyrShape(SimplexLikeShape):
    """The pyramid: square base at z = -1, apex (0, 0, 1)
    (pyfr/shapes.py:573-635); its solution space holds modes of total
    degree up to twice the order."""
    name = 'pyr'
    ndims = 3
    space_degree = 2

    faces = [
        ('quad', lambda s, t: (s, t, -1), (0, 0, -1)),
        ('tri', lambda s, t: (s + (t + 1)/2, (t - 1)/2, t), (0, -1, 0.5)),
        ('tri', lambda s, t: ((1 - t)/2, -s - (t + 1)/2, t), (1, 0, 0.5)),
        ('tri', lambda s, t: (-s - (t + 1)/2, (1 - t)/2, t), (0, 1, 0.5)),
        ('tri', lambda s, t: ((t - 1)/2, s + (t + 1)/2, t), (-1, 0, 0.5)),
    ]

    def _solution_basis(self):
        return PyrBasis(self.order, self.upts)


# Vertices of the linear elements, in the reference's order (std_ele(1)
# of pyfr/shapes.py)
VERTICES = {
    'quad': [(-1, -1), (1, -1), (-1, 1), (1, 1)],
    'hex': [(-1, -1, -1), (1, -1, -1), (-1, 1, -1), (1, 1, -1),
            (-1, -1, 1), (1, -1, 1), (-1, 1, 1), (1, 1, 1)],
    'tri': [(-1, -1), (1, -1), (-1, 1)],
    'tet': [(-1, -1, -1), (1, -1, -1), (-1, 1, -1), (-1, -1, 1)],
    'pri': [(-1, -1, -1), (1, -1, -1), (-1, 1, -1),
            (-1, -1, 1), (1, -1, 1), (-1, 1, 1)],
    'pyr': [(-1, -1, -1), (1, -1, -1), (-1, 1, -1), (1, 1, -1), (0, 0, 1)],
}

# Element type from (ndims, number of vertices)
ETYPE_OF = {(2, 4): 'quad', (3, 8): 'hex', (2, 3): 'tri', (3, 4): 'tet',
            (3, 6): 'pri', (3, 5): 'pyr'}


def _simplex_bary(x):
    """Barycentric coordinates of the reference triangle/tetrahedron:
    vertex 0 then one per coordinate; with their constant gradients."""
    nd = x.shape[1]
    lam = np.empty((len(x), nd + 1))
    lam[:, 0] = -(x.sum(axis=1) + nd - 2)/2
    lam[:, 1:] = (1 + x)/2
    grad = np.zeros((nd, nd + 1))
    grad[:, 0] = -0.5
    grad[np.arange(nd), np.arange(1, nd + 1)] = 0.5
    return lam, grad


def linear_shape_fn(etype, x):
    """Shape functions (npts, nverts) of the linear element of ``etype``
    (the interpolation expressions of pyfr/shapes.py)."""
    x = np.asarray(x, dtype=float)
    if etype in ('quad', 'hex'):
        v = np.array(VERTICES[etype], dtype=float)
        return np.prod(1 + x[:, None, :]*v[None, :, :], axis=2)/len(v)
    if etype in ('tri', 'tet'):
        return _simplex_bary(x)[0]
    if etype == 'pri':
        lam, _ = _simplex_bary(x[:, :2])
        z = x[:, 2:3]
        return np.hstack([lam*(1 - z)/2, lam*(1 + z)/2])
    if etype == 'pyr':
        return _pyr_shape(x)[0]
    raise ValueError(etype)


def linear_shape_jac(etype, x):
    """Reference gradients (npts, ndims, nverts) of the linear shape
    functions of ``etype`` (the Jacobian expressions of pyfr/shapes.py)."""
    x = np.atleast_2d(np.asarray(x, dtype=float))
    npt, nd = x.shape
    if etype in ('quad', 'hex'):
        v = np.array(VERTICES[etype], dtype=float)
        out = np.empty((npt, nd, len(v)))
        for i in range(nd):
            t = np.ones((npt, len(v)))
            for d in range(nd):
                t = t*(v[None, :, d] if d == i else 1 + x[:, None, d]*v[None, :, d])
            out[:, i] = t/len(v)
        return out
    if etype in ('tri', 'tet'):
        _, g = _simplex_bary(x)
        return np.broadcast_to(g, (npt,) + g.shape).copy()
    if etype == 'pri':
        lam, g = _simplex_bary(x[:, :2])
        z = x[:, 2][:, None]
        out = np.empty((npt, 3, 6))
        for i in range(2):
            out[:, i, :3] = g[i]*(1 - z)/2
            out[:, i, 3:] = g[i]*(1 + z)/2
        out[:, 2, :3] = -lam/2
        out[:, 2, 3:] = lam/2
        return out
    if etype == 'pyr':
        return _pyr_shape(x)[1]
    raise ValueError(etype)


def _pyr_shape(x):
    """Shape functions and their reference gradients of the linear pyramid
    (the space {1, x, y, z, xy} of the reference's interpolation and
    Jacobian expressions, pyfr/shapes.py:590-616): a base vertex
    (xv, yv, -1) has N = (2 (1 + xv x)(1 + yv y) - (1 + z))/8, the apex
    N = (1 + z)/2.  The map is affine when the base is a parallelogram."""
    npt = len(x)
    v = np.array(VERTICES['pyr'][:4], dtype=float)
    px, py, pz = x[:, 0:1], x[:, 1:2], x[:, 2:3]
    fx, fy = 1 + v[None, :, 0]*px, 1 + v[None, :, 1]*py
    N = np.hstack([(2*fx*fy - (1 + pz))/8, (1 + pz)/2])
    dN = np.empty((npt, 3, 5))
    dN[:, 0, :4] = v[None, :, 0]*fy/4
    dN[:, 1, :4] = v[None, :, 1]*fx/4
    dN[:, 2, :4] = -1/8
    dN[:, 0, 4] = dN[:, 1, 4] = 0
    dN[:, 2, 4] = 1/2
    return N, dN


SHAPES = {'quad': QuadShape, 'hex': HexShape, 'tri': TriShape,
          'tet': TetShape, 'pri': PriShape, 'pyr': PyrShape}


def get_shape(name, order, upts_rule='gauss-legendre',
              fpts_rule='gauss-legendre'):
    """Shape ``name`` of order ``order``; ``fpts_rule`` names the flux
    point rule of every face kind, or maps face kinds to rules."""
    try:
        cls = SHAPES[name]
    except KeyError:
        raise ValueError(f'Unsupported element type {name!r}') from None
    return cls(order, upts_rule, fpts_rule)


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
