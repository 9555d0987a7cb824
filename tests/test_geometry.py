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
