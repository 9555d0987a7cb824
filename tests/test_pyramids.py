"""Pyramids against the reference's own pyramid (``pyfr/shapes.py:573-635``,
``pyfr/polys.py:333-402``, ``pyfr/quadrules/pyr``), and the box where
hexahedra meet tetrahedra through pyramids.

* The layered Gauss-Legendre and Gauss-Legendre-Lobatto point sets equal
  the reference's tables; every operator (M0-M6 and the combined
  expressions) equals the reference's at orders 1-4 (1e-12 of the
  matrix's largest entry; 5e-12 at order 4, where the two constructions
  round differently at that level).
* The pyramid's modes are orthonormal on the element and span the
  reference's space (the projection of the reference's nodal basis).
* Geometry of pyramids whose bases are not parallelograms (maps that are
  not affine) equals the reference's: 1/|J|, metric terms and normals.
* The hexahedron-pyramid-tetrahedron box: every face pairs, the geometry
  and face-point order equal the reference's elements', the oracle's
  pairing is the reference's, and the oracle keeps a free stream with
  the reference's operators."""
import numpy as np
import pytest

from pyfr_gb300.inifile import Inifile
from pyfr_gb300.shapes import get_shape
from tests.oracle_util import basis_of, ops_from_golden

GAS = dict(gamma=1.4, mu=0.01, Pr=0.72, **{'ldg-beta': 0.5, 'ldg-tau': 0.1})
FPTS = {'quad': 'gauss-legendre', 'tri': 'alpha-opt'}
UPTS = {'hex': 'gauss-legendre', 'pyr': 'gauss-legendre', 'tet': 'alpha-opt'}
CASES = [(p, r) for p in (1, 2, 3, 4)
         for r in ('gauss-legendre', 'gauss-legendre-lobatto')]


@pytest.mark.parametrize('order,upts', CASES)
def test_pyramid_operators_match_reference(golden, order, upts):
    ref = golden['operators']
    key = f'pyr_p{order}_{upts}'
    s = get_shape('pyr', order, upts, FPTS)
    np.testing.assert_allclose(s.upts, ref[f'{key}/upts'], atol=1e-15)
    np.testing.assert_allclose(s.fpts, ref[f'{key}/fpts'], atol=1e-15)
    np.testing.assert_array_equal(s.nfacefpts, ref[f'{key}/nfacefpts'])
    np.testing.assert_array_equal(s.norm_fpts, ref[f'{key}/norm_fpts'])
    exprs = {'M132': 'M1 - M3*M2', 'M460': 'M4 - M6*M0'}
    # Relative to the matrix's largest entry: 1e-12, and 5e-12 at order 4,
    # where the two constructions round differently at that level
    tol = 5e-12 if order == 4 else 1e-12
    for m in ('m0', 'm1', 'm2', 'm3', 'm4', 'm6', 'M132', 'M460'):
        mine = s.opmat(exprs[m]) if m in exprs else getattr(s, m)
        r = ref[f'{key}/{m}']
        np.testing.assert_allclose(mine, r, rtol=0,
                                   atol=tol*np.abs(r).max(), err_msg=m)


@pytest.mark.parametrize('order', [1, 2, 3, 4])
def test_pyramid_basis_orthonormal_and_complete(order):
    from pyfr_gb300.polys import PyrBasis
    from pyfr_gb300.quadrules import point_set, pyr_gauss
    b = PyrBasis(order, point_set('pyr', 'gauss-legendre', order))
    qp, qw = pyr_gauss(4*order)
    ob = b.ortho_basis_at(qp)
    np.testing.assert_allclose((ob*qw) @ ob.T, np.eye(len(ob)), atol=1e-13)
    # Members of the space are reproduced by their projection: the mode
    # i = j = p, k = 0, (1 - z)^(2p) P_p(2x/(1 - z)) P_p(2y/(1 - z)) (a
    # polynomial of degree 2p), x y, z^p and x z^(p - 1)
    from numpy.polynomial.legendre import legval
    x, y, z = qp.T
    w = 1 - z
    c = [0]*order + [1]
    top = w**(2*order)*legval(2*x/w, c)*legval(2*y/w, c)
    for f in (top, x*y, z**order, x*z**(order - 1)):
        c = ob @ (qw*f)
        np.testing.assert_allclose(c @ ob, f, atol=1e-11)


def test_pyramid_quadrature_exact():
    from pyfr_gb300.quadrules import pyr_gauss
    qp, qw = pyr_gauss(9)
    x, y, z = qp.T
    assert abs(qw.sum() - 8/3) < 1e-14
    # int z^k over the pyramid: int_-1^1 z^k (1 - z)^2 dz
    for k in range(8):
        exact = np.polynomial.polynomial.polyint(
            np.polynomial.polynomial.polymul([0]*k + [1], [1, -2, 1]))
        want = np.polynomial.polynomial.polyval(1, exact) - \
            np.polynomial.polynomial.polyval(-1, exact)
        assert abs((qw*z**k).sum() - want) < 1e-13
    # int x^2 y^2 = int_-1^1 (2 h^3/3)^2 dz with h = (1 - z)/2
    want = 4/9*2/7
    assert abs((qw*x*x*y*y).sum() - want) < 1e-14


def _elements(g, etype, spts):
    from pyfr_gb300.solvers.elements import EulerElements
    cfg = Inifile()
    cfg.set('solver', 'order', 3)
    cfg.set('constants', 'gamma', 1.4)
    cfg.set('solver-elements-pyr', 'soln-pts', 'gauss-legendre')
    for k in [k for k in g if k.startswith('icexpr/')]:
        cfg.set('soln-ics', k.split('/')[1], str(g[k]))
    return EulerElements(etype, spts, cfg)


def _check_geometry(e, g, pre=''):
    np.testing.assert_allclose(e.ploc_at_np('upts'), g[f'{pre}ploc_upts'],
                               atol=1e-13)
    np.testing.assert_allclose(e.rcpdjac_at_np('upts'),
                               g[f'{pre}rcpdjac_upts'], rtol=1e-11)
    np.testing.assert_allclose(e.smat_at_np('upts'), g[f'{pre}smat_upts'],
                               rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(e._pnorm_fpts, g[f'{pre}pnorm_fpts'],
                               rtol=1e-11, atol=1e-13)


def test_skewed_pyramid_geometry_matches_reference(golden):
    """Pyramids with random vertices: the map is not affine (the xy term
    of the linear pyramid), so the metric terms vary over the element."""
    from pyfr_gb300.backend.pointwise import affine, linear_metrics
    g = golden['geometry_pyrskew_p3']
    e = _elements({}, 'pyr', g['spts'])
    _check_geometry(e, g)
    sm, _ = linear_metrics(g['spts'].transpose(0, 2, 1), e.basis.upts)
    assert not affine(sm)


def test_oracle_pyramid_geometry_matches_reference(golden):
    from oracle.fr_oracle import linear_smats_djac
    g = golden['geometry_pyrskew_p3']
    s = get_shape('pyr', 3, 'gauss-legendre', FPTS)
    _, d = linear_smats_djac('pyr', g['spts'], s.upts)
    np.testing.assert_allclose(1/d, g['rcpdjac_upts'], rtol=1e-11)


@pytest.mark.parametrize('etype', ['hex', 'pyr', 'tet'])
def test_hexpyrtet_geometry_matches_reference(golden, etype):
    g = golden['geometry_hexpyrtet_p3']
    e = _elements(g, etype, g[f'{etype}/spts'])
    _check_geometry(e, g, f'{etype}/')
    for fi, sf in enumerate(e.srtd_face_fpts):
        np.testing.assert_array_equal(sf, g[f'{etype}/srtd_face_fpts/{fi}'])
    np.testing.assert_allclose(e.set_ics_from_cfg(), g[f'{etype}/ics'],
                               rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize('n', [2, 4])
def test_hexpyrtet_box_conforms(n):
    """Every face pairs with a face of its kind and centroid; hexahedra
    meet only hexahedra and pyramid bases, tetrahedra only tetrahedra and
    pyramid sides; volume is that of the box."""
    from pyfr_gb300.mesh import face_vertices, mixed_box
    from pyfr_gb300.quadrules import EXACT_RULES
    from pyfr_gb300.shapes import SHAPES, linear_shape_jac
    m = mixed_box(n, 0.0, 1.0, 'hex-pyr-tet')
    lhs, rhs = m.con
    nfaces = sum(v.shape[1]*len(SHAPES[k].faces) for k, v in m.spts.items())
    assert 2*len(lhs) == nfaces
    for a, b in zip(zip(lhs.etypes, lhs.eidxs, lhs.fidxs),
                    zip(rhs.etypes, rhs.eidxs, rhs.fidxs)):
        assert {a[0], b[0]} != {'hex', 'tet'}
        assert SHAPES[a[0]].faces[a[2]][0] == SHAPES[b[0]].faces[b[2]][0]
        va = m.spts[a[0]][face_vertices(a[0])[a[2]], a[1]]
        vb = m.spts[b[0]][face_vertices(b[0])[b[2]], b[1]]
        assert np.allclose(np.mod(va.mean(0) + 1e-9, 1.0),
                           np.mod(vb.mean(0) + 1e-9, 1.0))
    vol = 0
    for et, sp in m.spts.items():
        qp, qw = EXACT_RULES[et](2)
        J = np.einsum('piv,vej->pije', linear_shape_jac(et, qp), sp)
        d = np.linalg.det(J.transpose(0, 3, 1, 2))
        assert d.min() > 0
        vol += (qw[:, None]*d).sum()
    assert abs(vol - 1) < 1e-12
    assert {k: v.shape[1] for k, v in m.spts.items()} == \
        {'hex': n**3//2, 'pyr': 2*(n*n), 'tet': 2*(6*n**3//2 - 2*n*n)}


def _mixed_disc(golden, ns=False):
    from oracle.fr_oracle import MixedDiscretisation
    g = golden['geometry_hexpyrtet_p3']
    ops = golden['operators']
    keys = {'hex': 'hex_p3_gauss-legendre', 'pyr': 'pyr_p3_gauss-legendre',
            'tet': 'tet_p3_mixed'}
    parts = {}
    for et in ('hex', 'pyr', 'tet'):
        s = get_shape(et, 3, UPTS[et], FPTS)
        parts[et] = dict(ops=ops_from_golden(ops, keys[et], ns),
                         basis=basis_of(s), verts=g[f'{et}/spts'])
    return MixedDiscretisation(parts, g['lhs'], g['rhs'],
                               periods=(2.0,)*3), g


def test_hexpyrtet_oracle_pairing_is_the_references(golden):
    d, g = _mixed_disc(golden)
    srt = {et: [g[f'{et}/srtd_face_fpts/{f}']
                for f in range(len(e['facefpts']))] for et, e in d.p.items()}
    ref = set()
    for (tl, el, fl), (tr, er, fr) in zip(g['lhs'], g['rhs']):
        el, fl, er, fr = int(el), int(fl), int(er), int(fr)
        for a, b in zip(srt[tl][fl][el], srt[tr][fr][er]):
            ref.add((tl, int(a), el, tr, int(b), er))
    tl, fl, el = d.side['l']
    tr, fr, er = d.side['r']
    mine = {(d.etypes[a], int(b), int(c), d.etypes[x], int(y), int(z))
            for a, b, c, x, y, z in zip(tl, fl, el, tr, fr, er)}
    assert mine == ref


@pytest.mark.parametrize('ns', [False, True])
def test_hexpyrtet_free_stream(golden, ns):
    """A uniform state stays uniform.  (Discrete conservation, exact on the
    other element types, holds on pyramids only up to the flux points'
    quadrature of the face traces: the pyramid's modes reach degree 2p on
    its triangular faces, whose flux points integrate degree p exactly --
    the same in the reference, whose operators these are.)"""
    d, g = _mixed_disc(golden, ns)
    rhs = d.rhs_ns if ns else d.rhs_euler
    cons = np.array([1.2, 0.3, 0.6, 0.9, 3.0])
    u = {et: np.broadcast_to(cons[None, :, None],
                             (len(e['upts']), 5, e['neles'])).copy()
         for et, e in d.p.items()}
    assert max(np.abs(v).max() for v in rhs(u, GAS).values()) < 1e-11


@pytest.mark.parametrize('order', [1, 2, 3, 4])
def test_pyramid_box_free_stream(golden, order):
    """A periodic box of pyramids only (six per cell): the oracle with the
    reference's operators keeps a uniform state at every order."""
    from oracle.fr_oracle import MixedDiscretisation
    from pyfr_gb300.mesh import mixed_box
    mesh = mixed_box(2, -1.0, 1.0, 'pyr')
    sh = get_shape('pyr', order, 'gauss-legendre', FPTS)
    lhs, rhs = mesh.con
    d = MixedDiscretisation(
        {'pyr': dict(ops=ops_from_golden(golden['operators'],
                                         f'pyr_p{order}_gauss-legendre', True),
                     basis=basis_of(sh), verts=mesh.spts['pyr'])},
        zip(lhs.etypes, lhs.eidxs, lhs.fidxs),
        zip(rhs.etypes, rhs.eidxs, rhs.fidxs), periods=mesh.periods)
    cons = np.array([1.2, 0.3, 0.6, 0.9, 3.0])
    u = {'pyr': np.broadcast_to(cons[None, :, None],
                                (sh.nupts, 5, 48)).copy()}
    assert np.abs(d.rhs_euler(u, GAS)['pyr']).max() < 1e-11
    assert np.abs(d.rhs_ns(u, GAS)['pyr']).max() < 1e-11


@pytest.mark.parametrize('order', [1, 2, 3, 4])
def test_pyramid_modal_basis_is_the_references(golden, order):
    """The modes the entropy filter and the shock sensor group by degree:
    orthonormalised in the reference's mode order, they are the reference's
    orthonormal pyramid modes, sign included (tests/golden/bases.npz)."""
    from pyfr_gb300.polys import modal_basis
    g = golden['bases']
    key = f'pyr_p{order}'
    s = get_shape('pyr', order, 'gauss-legendre', FPTS)
    np.testing.assert_allclose(s.upts, g[f'{key}/pts'], atol=1e-15)
    ub, modes, lower = modal_basis(s)
    assert [tuple(d) for d in g[f'{key}/degrees']] == list(modes)
    np.testing.assert_allclose(ub.vdm, g[f'{key}/vdm'], rtol=0,
                               atol=1e-12 if order < 4 else 1e-10)
    assert set(lower) < set(modes)
