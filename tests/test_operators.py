"""Operator matrices against the reference's own values."""
import numpy as np
import pytest

from pyfr_gb300.shapes import get_shape

CASES = [('quad', 2, 'gauss-legendre'), ('quad', 3, 'gauss-legendre'),
         ('quad', 4, 'gauss-legendre'), ('quad', 3, 'gauss-legendre-lobatto'),
         ('hex', 2, 'gauss-legendre'), ('hex', 3, 'gauss-legendre'),
         ('hex', 4, 'gauss-legendre')]


@pytest.mark.parametrize('etype,order,pts', CASES)
def test_operators_match_reference(golden, etype, order, pts):
    ref = golden['operators']
    key = f'{etype}_p{order}_{pts}'
    s = get_shape(etype, order, pts, pts)

    np.testing.assert_allclose(s.upts, ref[f'{key}/upts'], atol=1e-14)
    np.testing.assert_allclose(s.fpts, ref[f'{key}/fpts'], atol=1e-14)
    np.testing.assert_array_equal(s.norm_fpts, ref[f'{key}/norm_fpts'])
    np.testing.assert_array_equal(s.nfacefpts, ref[f'{key}/nfacefpts'])

    for m in ('m0', 'm1', 'm2', 'm3', 'm4', 'm6'):
        np.testing.assert_allclose(getattr(s, m), ref[f'{key}/{m}'],
                                   rtol=0, atol=1e-11, err_msg=m)
    np.testing.assert_allclose(s.opmat('M1 - M3*M2'), ref[f'{key}/M132'],
                               rtol=0, atol=1e-11)
    np.testing.assert_allclose(s.opmat('M4 - M6*M0'), ref[f'{key}/M460'],
                               rtol=0, atol=1e-11)


@pytest.mark.parametrize('etype,order,pts', CASES)
def test_sparsity_pattern_matches_reference(golden, etype, order, pts):
    # Exact zeros drive the sparse operator kernels: patterns must agree
    ref = golden['operators']
    key = f'{etype}_p{order}_{pts}'
    s = get_shape(etype, order, pts, pts)
    for m, e in (('m0', 'M0'), ('m3', 'M3'), ('M132', 'M1 - M3*M2'),
                 ('M460', 'M4 - M6*M0'), ('m6', 'M6')):
        np.testing.assert_array_equal(s.opmat(e) != 0, ref[f'{key}/{m}'] != 0)


def test_reference_golden_file(golden):
    # pyfr/tests/test_ele_mats.py: hex p=3 Gauss-Legendre m0..m3
    ref = golden['operators']
    s = get_shape('hex', 3)
    for m in ('m0', 'm1', 'm2', 'm3'):
        assert np.allclose(getattr(s, m), ref[f'refgolden/hex_p3/{m}'])


def test_opmat_rejects_bad_expression():
    s = get_shape('quad', 2)
    with pytest.raises(ValueError):
        s.opmat('M0.__class__')


# Simplex and prism shapes: the reference's named 'alpha-opt' point sets
# are computed here (warp and blend), listed in lattice order; the
# triangle table of the reference lists the same points grouped by
# symmetry orbit.  Points are matched by coordinates, then every operator
# must agree entry for entry under that permutation.
SIMPLEX = [('tri', p, 'alpha-opt', 'gauss-legendre') for p in (2, 3, 4)] + \
    [('tet', p, 'alpha-opt', {'tri': 'alpha-opt'}) for p in (2, 3, 4)] + \
    [('pri', p, 'alpha-opt~gauss-legendre-lobatto',
      {'tri': 'alpha-opt', 'quad': 'gauss-legendre'}) for p in (2, 3, 4)]


def _perm(mine, ref, tol=1e-13):
    d = np.linalg.norm(mine[None, :, :] - ref[:, None, :], axis=2)
    idx = d.argmin(axis=1)
    assert d[np.arange(len(ref)), idx].max() < tol
    assert len(set(idx)) == len(ref)
    return idx


@pytest.mark.parametrize('etype,order,upts,fpts', SIMPLEX)
def test_simplex_operators_match_reference(golden, etype, order, upts, fpts):
    ref = golden['operators']
    key = f'{etype}_p{order}_{upts}'
    s = get_shape(etype, order, upts, fpts)
    pu = _perm(s.upts, ref[f'{key}/upts'])
    # Flux points on face edges appear once per face: match face by face
    pf = np.concatenate([np.array(f)[_perm(s.fpts[f], ref[f'{key}/fpts'][f])]
                         for f in s.facefpts])
    np.testing.assert_array_equal(s.nfacefpts, ref[f'{key}/nfacefpts'])
    np.testing.assert_array_equal(s.norm_fpts[pf], ref[f'{key}/norm_fpts'])

    # Operators over (dim, point) index pairs order them dim-major
    nd = s.ndims
    pdu = (np.arange(nd)[:, None]*s.nupts + pu[None, :]).ravel()
    cases = {'m0': (pf, pu), 'm1': (pu, pdu), 'm2': (pf, pdu),
             'm3': (pu, pf), 'm4': (pdu, pu), 'm6': (pdu, pf),
             'M132': (pu, pdu), 'M460': (pdu, pu)}
    exprs = {'M132': 'M1 - M3*M2', 'M460': 'M4 - M6*M0'}
    for m, (r, c) in cases.items():
        mine = s.opmat(exprs[m]) if m in exprs else getattr(s, m)
        np.testing.assert_allclose(mine[np.ix_(r, c)], ref[f'{key}/{m}'],
                                   rtol=0, atol=1e-11, err_msg=m)


@pytest.mark.parametrize('etype', ['quad', 'hex'])
def test_antialias_operators_match_reference(golden, etype):
    """Flux anti-aliasing: interpolation to the quadrature points (M7) and
    the L2 projection back (M9), default Gauss-Legendre (p+2)^d rule."""
    ref = golden['operators']
    key = f'{etype}_p3_aa'
    s = get_shape(etype, 3)
    np.testing.assert_allclose(s.qpts, ref[f'{key}/qpts'], atol=1e-14)
    np.testing.assert_allclose(s.m7, ref[f'{key}/m7'], rtol=0, atol=1e-11)
    np.testing.assert_allclose(s.m9, ref[f'{key}/m9'], rtol=0, atol=1e-11)
    np.testing.assert_allclose(s.opmat('(M1 - M3*M2)*M9'),
                               ref[f'{key}/M1329'], rtol=0, atol=1e-11)


@pytest.mark.parametrize('kind', ['tri', 'tet', 'pri'])
@pytest.mark.parametrize('order', [1, 2, 3, 4])
def test_simplex_ortho_basis_matches_reference(kind, order):
    """The collapsed-coordinate orthonormal bases (degree tuples, order and
    sign of the modes) against the reference's at its solution points
    (tests/golden/bases.npz, made by tests/golden/make_golden.py)."""
    from pathlib import Path
    from pyfr_gb300.polys import SimplexOrthoBasis
    g = np.load(Path(__file__).parent / 'golden' / 'bases.npz')
    key = f'{kind}_p{order}'
    b = SimplexOrthoBasis(kind, order, g[f'{key}/pts'])
    assert [tuple(d) for d in g[f'{key}/degrees']] == b.degrees
    np.testing.assert_allclose(b.vdm, g[f'{key}/vdm'], rtol=0, atol=1e-12)


@pytest.mark.parametrize('name', ['quad', 'hex'])
@pytest.mark.parametrize('order', [2, 3])
def test_surface_antialiasing_operators(name, order):
    """Surface-flux anti-aliasing: flux points at the face quadrature
    points, M0 there and M3 with the L2 projection onto the face bases,
    against the reference's (tests/golden/surf_flux.npz), up to the order
    of the points."""
    from pathlib import Path
    from pyfr_gb300.quadrules import tensor_rule
    g = np.load(Path(__file__).parent / 'golden' / 'surf_flux.npz')
    key = f'{name}_p{order}'
    s = get_shape(name, order)
    nd = s.ndims
    fk = 'line' if nd == 2 else 'quad'
    s.set_surf_rules({fk: tensor_rule('gauss-legendre', order + 2, nd - 1)})
    rf = g[f'{key}/fpts']
    perm = [int(np.argmin(np.linalg.norm(s.fpts - p, axis=1))) for p in rf]
    assert sorted(perm) == list(range(len(rf)))
    np.testing.assert_allclose(s.fpts[perm], rf, atol=1e-14)
    np.testing.assert_allclose(s.m0[perm], g[f'{key}/m0'], atol=1e-12)
    np.testing.assert_allclose(s.m3[:, perm], g[f'{key}/m3'], atol=1e-12)
