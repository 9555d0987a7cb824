"""Element geometry, face flux-point ordering and initial conditions against
values computed by the reference's own element classes on perturbed
(non-affine) periodic meshes."""
import numpy as np
import pytest

from pyfr_gb300.inifile import Inifile
from pyfr_gb300.solvers.elements import EulerElements, NavierStokesElements


def _elements(g, etype):
    cfg = Inifile()
    cfg.set('solver', 'order', 3)
    cfg.set('constants', 'gamma', 1.4)
    for k in [k for k in g if k.startswith('icexpr/')]:
        cfg.set('soln-ics', k.split('/')[1], str(g[k]))
    cls = EulerElements if etype == 'quad' else NavierStokesElements
    return cls(etype, g['spts'], cfg)


@pytest.mark.parametrize('case,etype', [('quad_p3', 'quad'), ('hex_p3', 'hex')])
def test_geometry_matches_reference(golden, case, etype):
    g = golden[f'geometry_{case}']
    e = _elements(g, etype)

    np.testing.assert_allclose(e.basis.upts, g['upts'], atol=1e-14)
    np.testing.assert_allclose(e.ploc_at_np('upts'), g['ploc_upts'], atol=1e-13)
    np.testing.assert_allclose(e.rcpdjac_at_np('upts'), g['rcpdjac_upts'],
                               rtol=1e-11)
    np.testing.assert_allclose(e.smat_at_np('upts'), g['smat_upts'],
                               rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(e._pnorm_fpts, g['pnorm_fpts'], rtol=1e-11,
                               atol=1e-13)


@pytest.mark.parametrize('case,etype', [('quad_p3', 'quad'), ('hex_p3', 'hex')])
def test_face_point_order_matches_reference(golden, case, etype):
    g = golden[f'geometry_{case}']
    e = _elements(g, etype)
    for fi, sf in enumerate(e.srtd_face_fpts):
        np.testing.assert_array_equal(sf, g[f'srtd_face_fpts/{fi}'])


@pytest.mark.parametrize('case,etype', [('quad_p3', 'quad'), ('hex_p3', 'hex')])
def test_initial_conditions_match_reference(golden, case, etype):
    g = golden[f'geometry_{case}']
    e = _elements(g, etype)
    np.testing.assert_allclose(e.set_ics_from_cfg(), g['ics'], rtol=1e-13)


MIXED = [('hexpri_p3', 'hex'), ('hexpri_p3', 'pri'), ('pritet_p3', 'pri'),
         ('pritet_p3', 'tet')]


def _mixed_elements(g, etype):
    cfg = Inifile()
    cfg.set('solver', 'order', 3)
    cfg.set('constants', 'gamma', 1.4)
    for k in [k for k in g if k.startswith('icexpr/')]:
        cfg.set('soln-ics', k.split('/')[1], str(g[k]))
    return EulerElements(etype, g[f'{etype}/spts'], cfg)


@pytest.mark.parametrize('case,etype', MIXED)
def test_mixed_geometry_matches_reference(golden, case, etype):
    """Hexahedra, prisms and tetrahedra of perturbed conforming mixed
    meshes (the reference given this package's point sets literally)."""
    g = golden[f'geometry_{case}']
    e = _mixed_elements(g, etype)
    np.testing.assert_allclose(e.ploc_at_np('upts'), g[f'{etype}/ploc_upts'],
                               atol=1e-13)
    np.testing.assert_allclose(e.rcpdjac_at_np('upts'),
                               g[f'{etype}/rcpdjac_upts'], rtol=1e-11)
    np.testing.assert_allclose(e.smat_at_np('upts'), g[f'{etype}/smat_upts'],
                               rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(e._pnorm_fpts, g[f'{etype}/pnorm_fpts'],
                               rtol=1e-11, atol=1e-13)
    for fi, sf in enumerate(e.srtd_face_fpts):
        np.testing.assert_array_equal(sf, g[f'{etype}/srtd_face_fpts/{fi}'])
    np.testing.assert_allclose(e.set_ics_from_cfg(), g[f'{etype}/ics'],
                               rtol=1e-13)


@pytest.mark.parametrize('etype', ['pri', 'tet'])
def test_mixed_operators_match_reference(golden, etype):
    from pyfr_gb300.shapes import get_shape
    ref = golden['operators']
    key = f'{etype}_p3_mixed'
    upts = {'pri': 'alpha-opt~gauss-legendre-lobatto', 'tet': 'alpha-opt'}
    s = get_shape(etype, 3, upts[etype],
                  {'tri': 'alpha-opt', 'quad': 'gauss-legendre'})
    np.testing.assert_allclose(s.upts, ref[f'{key}/upts'], atol=1e-15)
    np.testing.assert_allclose(s.fpts, ref[f'{key}/fpts'], atol=1e-15)
    for m, e in (('m0', 'M0'), ('m3', 'M3'), ('M132', 'M1 - M3*M2'),
                 ('M460', 'M4 - M6*M0'), ('m6', 'M6')):
        np.testing.assert_allclose(s.opmat(e), ref[f'{key}/{m}'], rtol=0,
                                   atol=1e-11, err_msg=m)


def test_mixed_mesh_connectivity():
    """Every face pairs with one face of the same kind and the same
    centroid (modulo the periods), for meshes down to two cells per
    direction."""
    from pyfr_gb300.mesh import face_vertices, mixed_box
    from pyfr_gb300.shapes import SHAPES
    for kinds in ('hex-pri', 'pri-tet'):
        for n in (2, 3):
            m = mixed_box(n, 0.0, 1.0, kinds)
            lhs, rhs = m.con
            nfaces = sum(v.shape[1]*len(SHAPES[k].faces)
                         for k, v in m.spts.items())
            assert 2*len(lhs) == nfaces
            for a, b in zip(zip(lhs.etypes, lhs.eidxs, lhs.fidxs),
                            zip(rhs.etypes, rhs.eidxs, rhs.fidxs)):
                ka = SHAPES[a[0]].faces[a[2]][0]
                kb = SHAPES[b[0]].faces[b[2]][0]
                assert ka == kb
                va = m.spts[a[0]][face_vertices(a[0])[a[2]], a[1]]
                vb = m.spts[b[0]][face_vertices(b[0])[b[2]], b[1]]
                ca = np.mod(va.mean(0) + 1e-9, 1.0)
                cb = np.mod(vb.mean(0) + 1e-9, 1.0)
                assert np.allclose(ca, cb)


def test_affine_elements_detected():
    """Metric terms are kept per element exactly when every element's
    Jacobian is constant: uniform boxes, skewed parallelepipeds and linear
    tetrahedra; not a box with one moved interior vertex, not prisms."""
    from pyfr_gb300.backend.pointwise import affine, linear_metrics
    from pyfr_gb300.mesh import mixed_box, periodic_box
    from pyfr_gb300.shapes import get_shape

    upts = get_shape('hex', 3, 'gauss-legendre', 'gauss-legendre').upts
    m = periodic_box('hex', 4, -np.pi, np.pi)
    v = m.spts['hex'].transpose(0, 2, 1)          # (nverts, ndims, neles)
    assert affine(linear_metrics(v, upts)[0])

    # A shear keeps elements affine; moving one vertex does not
    sv = v.copy()
    sv[:, 0] += 0.3*sv[:, 1]
    assert affine(linear_metrics(sv, upts)[0])
    sv[3, 1, 5] += 0.05
    assert not affine(linear_metrics(sv, upts)[0])

    mb = mixed_box(2, 0.0, 1.0, 'pri-tet')
    for et, want in (('tet', True), ('pri', None)):
        x = get_shape(et, 3, 'alpha-opt', 'alpha-opt').upts if et == 'tet' \
            else get_shape(et, 3, 'alpha-opt~gauss-legendre-lobatto',
                           'alpha-opt~gauss-legendre').upts
        got = affine(linear_metrics(mb.spts[et].transpose(0, 2, 1), x)[0])
        if want is not None:
            assert got == want
